// hb_dem.cu -- DEM (FP64) and LB-DEM coupling: one cooperative kernel per cycle.
//
// DEM::discreteElementStep (DEM.cpp:331-376) runs multiStep substeps of
//   [neighbour rebuild if maxDisp > 0.25 nebrRange] predict -> forces -> correct.
// Here every substep is "forces | correct + the NEXT substep's predictor" (the predictor
// depends only on the element's own corrected state, elmt.cpp:139-177), with the
// rebuild (cell sort in one block, candidate lists per particle) only when the device
// displacement trigger fired.  The element hydrodynamic-force reduction of the previous
// lattice step runs first and the coupling masks (LB.cpp:1921-2033) last, all in one
// cooperative launch separated by grid barriers: two kernels per cycle in total (this
// one and the lattice kernel) instead of one per phase.
//
// Contacts: every particle owns its candidate list (both directions).  A pair is always
// evaluated with I = min index, J = max index, so both owners compute bit-identical
// pair forces; each sums its own side in list order.  No floating-point atomics.
//
// Coupling: one CTA per particle (grid-stride) sweeps the particle's bounding box.
#include <cooperative_groups.h>
#include <cstdio>
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace cg = cooperative_groups;

namespace hb {

constexpr int DEM_MAX_CYL = 4;  // cylinders the DEM contacts handle

struct DemArgs {
    int E;
    double *x0, *x1, *x2, *x3, *x4, *x5;
    double *xp0, *xp1, *xp2, *xp3, *xp4, *xp5;
    double *w0, *w1, *w2, *w3, *w4, *w5;
    double *wp0, *wp1, *wp2, *wp3, *wp4, *wp5;
    double *q0, *q1, *q2, *q3, *q4, *q5;
    double *qp0, *qp1, *qp2, *qp3, *qp4, *qp5;
    double *wG, *wL, *wpG, *wpL;
    double *FH, *MH, *FP, *FW, *MP, *MW;
    double *fvol, *m, *I, *rad;
    // second copy of the predicted position, velocity and global spin (the fields a
    // contact partner reads): the single-barrier substep of plain spheres reads one copy
    // and predicts into the other, alternating by substep
    double *xq0, *xq1, *wqG;
    float* pf;         // [12E] FP32 centre, velocity, spin (+ pad) per particle
    const int* plain;  // 1: orientation fixed at identity (no quaternion rates)
    int *cell_of, *cell_cnt, *cell_start, *cell_fill, *cell_items;
    int *nbr, *nbr_cnt, *wall_of, *obj, *obj_cnt;
    double* npc;          // [4 E nbr_cap] constants of each candidate pair (single spheres)
    int nbr_cap;          // candidate partners kept per particle (hb_params.cap_neighbors)
    double *wrec, *orec;  // wall / object contact records of the current substep (7 doubles each)
    int* cyl_of;          // [E] first cylinder in range or -1 (DEM.cpp:1535-1550)
    int ncyl;
    double cp1[DEM_MAX_CYL][3], cnax[DEM_MAX_CYL][3], cR[DEM_MAX_CYL], comg[DEM_MAX_CYL][3];
    int cmov[DEM_MAX_CYL];
    double* scal;
    int* contacts;
    double* partial;
    unsigned int* done;
    int ncells, nC0, nC1, nC2;
    double cw0, cw1, cw2, nebrRange, trigger, dt;
    // Gear coefficients (elmt.cpp:139-254): c_k = dt^k / k!, and the corrector weights of
    // the position/orientation (2nd order) and spin (1st order) chains, computed once on
    // the host with the same expressions (FP64 divisions are costly on this part's pipe)
    double gc[5], gc1[6], gc2[6];
    int nw;
    double wp[MAX_WALLS][3], wn[MAX_WALLS][3];
    int O;
    const double *ox0, *ox1, *orad;
    int model;
    double kn, damp, knConst, ksConst, viscTang, muPart, muWall, numVisc, demF[3];
    int* status;
    unsigned long long* total_contacts;
    // periodic faces: plane pl1 (point pp1, normal pn) and pl2 (point pp1 + v, normal -pn)
    // of each pair, and the shift v (pbc::setPlanes, utils.cpp:240-245)
    int npbc, gcap;
    double pp1[3][3], pp2[3][3], pn1[3][3], pn2[3][3], pv[3][3];
    int *gmeta, *gorig, *comp, *ccnt;
    double *gvec, *px;
    // per-particle path (periodic faces or multi-sphere elements): P standard particles,
    // element e owns efirst[e] .. efirst[e+1]-1
    int P, gen;
    int *pkey, *ecomp, *eccnt;
    const int *efirst, *esize;
    const double* proto;
    double *ppos, *pvel, *prv, *pF, *pcen;
};

struct V {
    double x, y, z;
};
__device__ __forceinline__ V ld3(const double* a, int E, int i) { return V{a[i], a[E + i], a[2 * E + i]}; }
__device__ __forceinline__ void st3(double* a, int E, int i, V v) {
    a[i] = v.x; a[E + i] = v.y; a[2 * E + i] = v.z;
}
__device__ __forceinline__ V add(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V sub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V mul(double s, V a) { return V{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V divs(V a, double s) { return V{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double nrm2(V a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V cross(V a, V b) {
    return V{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
struct Qt {
    double a, b, c, d;
};
__device__ __forceinline__ Qt ldq(const double* q, int E, int i) { return Qt{q[i], q[E + i], q[2 * E + i], q[3 * E + i]}; }
__device__ __forceinline__ void stq(double* q, int E, int i, Qt v) {
    q[i] = v.a; q[E + i] = v.b; q[2 * E + i] = v.c; q[3 * E + i] = v.d;
}
__device__ __forceinline__ Qt qmul(Qt p, Qt q) {  // vector.cpp:222-228, p.multiply(q)
    return Qt{q.a * p.a - q.b * p.b - q.c * p.c - q.d * p.d, q.a * p.b + q.b * p.a - q.c * p.d + q.d * p.c,
              q.a * p.c + q.b * p.d + q.c * p.a - q.d * p.b, q.a * p.d - q.b * p.c + q.c * p.b + q.d * p.a};
}
__device__ __forceinline__ Qt qadj(Qt p) { return Qt{p.a, -p.b, -p.c, -p.d}; }
__device__ __forceinline__ V project(V v, Qt q) {  // vector.cpp:364-370
    Qt r = qmul(qmul(q, Qt{0.0, v.x, v.y, v.z}), qadj(q));
    return V{r.b, r.c, r.d};
}
__device__ __forceinline__ Qt qaxpy(Qt a, Qt b, double s) { return Qt{a.a + b.a * s, a.b + b.b * s, a.c + b.c * s, a.d + b.d * s}; }

// Where the predicted position, velocity and global spin are read (r) and where the
// predictor writes the next substep's (w): the same arrays when a substep has a barrier
// between its force and corrector phases, alternate copies in the single-barrier substep.
struct PredBuf {
    const double *x0r, *x1r, *wGr;
    double *x0w, *x1w, *wGw;
};
__device__ __forceinline__ PredBuf pred_inplace(const DemArgs& a) {
    return PredBuf{a.xp0, a.xp1, a.wpG, a.xp0, a.xp1, a.wpG};
}
__device__ __forceinline__ PredBuf pred_alternate(const DemArgs& a, int par) {
    return par ? PredBuf{a.xq0, a.xq1, a.wqG, a.xp0, a.xp1, a.wpG} : PredBuf{a.xp0, a.xp1, a.wpG, a.xq0, a.xq1, a.wqG};
}

__device__ double normal_contact(const DemArgs& a, double overlap, double vn, double effRad, double effMass) {
    if (a.model == HB_HERTZIAN) {  // DEM.cpp:2142-2152
        const double kn = a.knConst * sqrt(effRad) * sqrt(overlap);
        const double gn = 2.0 * a.damp * sqrt(kn * effMass);
        return fmax(kn * overlap + (-gn * vn), 0.0);
    }
    const double el = a.kn * overlap;  // DEM.cpp:2153-2160
    const double gn = 2.0 * a.damp * sqrt(a.kn * effMass);
    return fmax(el + (-gn * vn), 0.0);
}
__device__ double tangential_contact(const DemArgs& a, double vt, double fn, double effRad, double effMass,
                                     double mu) {  // DEM.cpp:2176-2222
    const double ks = a.model == HB_HERTZIAN ? a.ksConst * sqrt(effRad) * pow(fabs(fn), 1.0 / 3.0) : a.kn;
    const double gs = 2.0 * a.viscTang * sqrt(effMass * ks);
    return fmin(gs * vt, mu * fn);
}

// ---- neighbour rebuild (DEM.cpp:1326-1533) -------------------------------------------

// single CTA: cell of every particle (linearizePosition, vector.cpp:147-149), counting
// sort into cells (counts, a block-wide scan, scatter), then ascending order inside each
// cell: the particles sorted by (cell, index)
// With periodic faces the table holds the ghosts too (after the elements, positions from
// the rebuild's px) and a particle's cell is the reference's linear index itself: a ghost
// above the last y cell row lands in row 0 of the next z slab, as in the reference's cell
// table, so the half-shell sweep below finds exactly the reference's pairs.  An index
// outside the table (the reference writes out of bounds there) flags an error.
__device__ __noinline__ void nl_cells_block(const DemArgs& a) {
    const int E = a.E, nc = a.ncells;
    const bool per = a.gen != 0;
    const int S = per ? a.P + a.gmeta[0] : E;
    const long long st = per ? (long long)a.P + a.gcap : E;
    const double* pos = per ? a.px : a.x0;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) { a.cell_cnt[c] = 0; a.cell_fill[c] = 0; }
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const V x{pos[i], pos[st + i], pos[2 * st + i]};
        const int c0 = (int)floor(x.x / a.cw0) + 1, c1 = (int)floor(x.y / a.cw1) + 2, c2 = (int)floor(x.z / a.cw2);
        int c = -1;
        if (per) {
            const long long L = c0 + (long long)a.nC0 * (c1 + (long long)a.nC1 * c2);  // vector.cpp:147-149
            if (L >= 0 && L < nc) c = (int)L;
        } else if (c0 >= 0 && c0 < a.nC0 && c1 >= 0 && c1 < a.nC1 && c2 >= 0 && c2 < a.nC2) {
            c = c0 + a.nC0 * (c1 + a.nC1 * c2);
        }
        if (c < 0) atomicOr(a.status + 2, 2);  // particle outside the box
        a.cell_of[i] = c;
        if (c >= 0) atomicAdd(a.cell_cnt + c, 1);
    }
    if (per)
        for (int i = threadIdx.x; i < a.P; i += blockDim.x) a.nbr_cnt[i] = 0;
    __syncthreads();
    {  // exclusive scan of the cell counts by the whole block, a chunk of blockDim cells at
       // a time (Hillis-Steele in shared memory), carrying the running total
        __shared__ int sc[256];
        __shared__ int carry;
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
            const int c = c0 + threadIdx.x;
            const int v = c < nc ? a.cell_cnt[c] : 0;
            sc[threadIdx.x] = v;
            __syncthreads();
            for (int off = 1; off < (int)blockDim.x; off <<= 1) {
                const int add = threadIdx.x >= (unsigned)off ? sc[threadIdx.x - off] : 0;
                __syncthreads();
                sc[threadIdx.x] += add;
                __syncthreads();
            }
            if (c < nc) a.cell_start[c] = carry + sc[threadIdx.x] - v;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) carry += sc[threadIdx.x];
            __syncthreads();
        }
        if (threadIdx.x == 0) a.cell_start[nc] = carry;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const int c = a.cell_of[i];
        if (c >= 0) a.cell_items[a.cell_start[c] + atomicAdd(a.cell_fill + c, 1)] = i;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {  // insertion sort per cell
        const int s = a.cell_start[c], e = a.cell_start[c + 1];
        for (int k = s + 1; k < e; ++k) {
            const int v = a.cell_items[k];
            int m = k - 1;
            while (m >= s && a.cell_items[m] > v) { a.cell_items[m + 1] = a.cell_items[m]; --m; }
            a.cell_items[m + 1] = v;
        }
    }
}

__device__ __noinline__ void nl_near_one(const DemArgs& a, int i);

// candidate list of every particle: all others within nebrRange in the 27 adjacent
// cells, then the walls, cylinder and objects in range
// The constants of candidate pair (i, j) in slot k of i's list, computed once per
// neighbour rebuild with the expressions particleParticleCollision evaluates at every
// contact (DEM.cpp:1801-1900, 2153-2222): effMass = mI mJ / (mI + mJ), effRad =
// rI rJ / (rI + rJ), and for the linear model the normal and tangential damping
// coefficients 2 damp sqrt(kn effMass), 2 viscTang sqrt(effMass kn).  Products and sums
// are commutative in IEEE arithmetic, so the values are those of the I = min(i, j)
// evaluation bit for bit; the contacts then take no FP64 division or square root for them.
__device__ __forceinline__ void pair_constants(const DemArgs& a, int i, int j, int k) {
    const long long st = (long long)a.E * a.nbr_cap, o = (long long)i * a.nbr_cap + k;
    const int I = min(i, j), J = max(i, j);
    const double mI = a.m[I], mJ = a.m[J], rI = a.rad[I], rJ = a.rad[J];
    const double effMass = mI * mJ / (mI + mJ);
    a.npc[o] = effMass;
    a.npc[st + o] = rI * rJ / (rI + rJ);
    a.npc[2 * st + o] = a.model == HB_HERTZIAN ? 0.0 : 2.0 * a.damp * sqrt(a.kn * effMass);
    a.npc[3 * st + o] = a.model == HB_HERTZIAN ? 0.0 : 2.0 * a.viscTang * sqrt(effMass * a.kn);
}

__device__ __noinline__ void nl_build_one(const DemArgs& a, int i) {
    const int E = a.E;
    const V xi = ld3(a.x0, E, i);
    const double r2 = a.nebrRange * a.nebrRange;
    int cnt = 0;
    const int c = a.cell_of[i];
    if (c >= 0) {
        const int c0 = c % a.nC0, c1 = (c / a.nC0) % a.nC1, c2 = c / (a.nC0 * a.nC1);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int n0 = c0 + dx, n1 = c1 + dy, n2 = c2 + dz;
                    if (n0 < 0 || n1 < 0 || n2 < 0 || n0 >= a.nC0 || n1 >= a.nC1 || n2 >= a.nC2) continue;
                    const int cc = n0 + a.nC0 * (n1 + a.nC1 * n2);
                    for (int k = a.cell_start[cc]; k < a.cell_start[cc + 1]; ++k) {
                        const int j = a.cell_items[k];
                        if (j == i) continue;
                        const V d = sub(ld3(a.x0, E, j), xi);
                        if (nrm2(d) < r2) {
                            if (cnt < a.nbr_cap) {
                                a.nbr[(long long)i * a.nbr_cap + cnt] = j;
                                if (a.npc) pair_constants(a, i, j, cnt);
                            }
                            ++cnt;
                        }
                    }
                }
    }
    if (cnt > a.nbr_cap) { atomicOr(a.status + 2, 1); cnt = a.nbr_cap; }
    a.nbr_cnt[i] = cnt;
    nl_near_one(a, i);
}

// first wall within range (DEM.cpp:1502-1511), first cylinder in range, objects in range
// (standard particles only, DEM.cpp:1496-1550)
__device__ __noinline__ void nl_near_one(const DemArgs& a, int i) {
    const int E = a.E;
    const long long st = (long long)a.P + a.gcap;
    const V xi = a.gen ? V{a.px[i], a.px[st + i], a.px[2 * st + i]} : ld3(a.x0, E, i);
    const double r2 = a.nebrRange * a.nebrRange;
    int wo = -1;
    for (int w = 0; w < a.nw; ++w) {
        const double d = a.wn[w][0] * (xi.x - a.wp[w][0]) + a.wn[w][1] * (xi.y - a.wp[w][1]) +
                         a.wn[w][2] * (xi.z - a.wp[w][2]);
        if (d < a.nebrRange) { wo = w; break; }
    }
    a.wall_of[i] = wo;
    int co = -1;  // evalNearCylinderTable: the first cylinder in range (cylinder::dist, utils.cpp:56-67)
    for (int c = 0; c < a.ncyl; ++c) {
        const V d = sub(xi, V{a.cp1[c][0], a.cp1[c][1], a.cp1[c][2]});
        const V nx{a.cnax[c][0], a.cnax[c][1], a.cnax[c][2]};
        const V dc = sub(mul(dot(d, nx), nx), d);
        if (a.cR[c] - sqrt(nrm2(dc)) < a.nebrRange) { co = c; break; }
    }
    a.cyl_of[i] = co;
    int oc = 0;
    for (int o = 0; o < a.O; ++o) {
        const V d = sub(xi, V{a.ox0[o], a.ox0[a.O + o], a.ox0[2 * a.O + o]});
        if (nrm2(d) < r2) {
            if (oc < OBJ_CAP) a.obj[(long long)i * OBJ_CAP + oc] = o;
            ++oc;
        }
    }
    if (oc > OBJ_CAP) { atomicOr(a.status + 2, 4); oc = OBJ_CAP; }
    a.obj_cnt[i] = oc;
}

// ---- periodic faces: shift, ghosts, half-shell sweep (DEM.cpp:1395-1494, 1554-1664) ------

__device__ __forceinline__ double plane_dist(const double* p, const double* n, V x) {  // wall::dist, utils.cpp:14-17
    return n[0] * (x.x - p[0]) + n[1] * (x.y - p[1]) + n[2] * (x.z - p[2]);
}

// exclusive prefix sum of v over the block (blockDim.x a multiple of 32, at most 1024);
// every thread of the block must call it
__device__ int block_scan(int v, int& total) {
    __shared__ int wsum[32];
    __shared__ int tot;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < nw; ++k) { const int t = wsum[k]; wsum[k] = run; run += t; }
        tot = run;
    }
    __syncthreads();
    const int r = wsum[w] + x - v;
    total = tot;
    __syncthreads();
    return r;
}

// side of face pair b that element n's centre copies to: +1 near pl1 (copied by +v), -1
// near pl2 (by -v), 0 neither; pl1 is tested first (DEM.cpp:1596-1616)
__device__ __forceinline__ int ghost_side(const DemArgs& a, int b, V x) {
    if (plane_dist(a.pp1[b], a.pn1[b], x) < a.nebrRange) return 1;
    if (plane_dist(a.pp2[b], a.pn2[b], x) < a.nebrRange) return -1;
    return 0;
}

// corrected centre of standard particle p (particle::updateCorrected, elmt.cpp:276-290)
__device__ __forceinline__ V part_pos_corr(const DemArgs& a, int p) {
    const int E = a.E, e = a.pkey[p];
    const V x = ld3(a.x0, E, e);
    if (a.esize[e] <= 1) return x;
    const V pr{a.proto[p], a.proto[a.P + p], a.proto[2 * a.P + p]};
    return add(x, mul(a.rad[e], project(pr, ldq(a.q0, E, e))));
}

// One block: pbcShift (elements whose centre left through a face move by the shift;
// elmt::translate moves x0 and xp0, elmt.cpp:256-259), the particles from their elements,
// then createGhosts: one ghost per (face pair, particle) whose centre is within
// nebrRange of a face, face pairs outer and particles inner, then one corner ghost per
// two ghosts of the same particle, ordered by the first ghost's index and then the
// second's.  Ghost g is particle P + g, like the reference's particles list; px holds
// every particle's centre, and each element lists its ghosts in creation order (the
// reference appends them to the element's components).
__device__ __noinline__ void ghosts_block(const DemArgs& a) {
    const int E = a.E, P = a.P;
    const long long st = (long long)P + a.gcap;
    for (int n = threadIdx.x; n < E; n += blockDim.x) {
        V x = ld3(a.x0, E, n), xp = ld3(a.xp0, E, n);
        for (int b = 0; b < a.npbc; ++b) {
            const double ld = plane_dist(a.pp1[b], a.pn1[b], x), rd = plane_dist(a.pp2[b], a.pn2[b], x);
            const V v{a.pv[b][0], a.pv[b][1], a.pv[b][2]};
            if (ld < 0.0) { x = add(x, v); xp = add(xp, v); }
            if (rd < 0.0) { const V mv = mul(-1.0, v); x = add(x, mv); xp = add(xp, mv); }
        }
        st3(a.x0, E, n, x);
        st3(a.xp0, E, n, xp);
        a.eccnt[n] = 0;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const V x = part_pos_corr(a, p);
        a.px[p] = x.x; a.px[st + p] = x.y; a.px[2 * st + p] = x.z;
        a.ccnt[p] = 0;
    }
    __syncthreads();
    int total = 0;
    for (int b = 0; b < a.npbc; ++b) {  // face ghosts
        for (int n0 = 0; n0 < P; n0 += blockDim.x) {
            const int n = n0 + threadIdx.x;
            const int sd = n < P ? ghost_side(a, b, V{a.px[n], a.px[st + n], a.px[2 * st + n]}) : 0;
            int sum;
            const int k = block_scan(sd != 0, sum);
            if (sd) {
                const int g = total + k;
                a.gorig[g] = n;
                a.pkey[P + g] = a.pkey[n];
                for (int q = 0; q < 3; ++q) a.gvec[(long long)q * a.gcap + g] = sd > 0 ? a.pv[b][q] : -1.0 * a.pv[b][q];
                a.comp[6 * n + a.ccnt[n]++] = P + g;
            }
            total += sum;
        }
    }
    for (int b1 = 0; b1 < a.npbc; ++b1) {  // corner ghosts
        for (int n0 = 0; n0 < P; n0 += blockDim.x) {
            const int n = n0 + threadIdx.x;
            int sd[3] = {0, 0, 0}, cnt = 0;
            if (n < P) {
                const V x{a.px[n], a.px[st + n], a.px[2 * st + n]};
                for (int b = 0; b < a.npbc; ++b) sd[b] = ghost_side(a, b, x);
                if (sd[b1])
                    for (int b2 = b1 + 1; b2 < a.npbc; ++b2) cnt += sd[b2] != 0;
            }
            int sum;
            const int k = block_scan(cnt, sum);
            if (cnt) {
                int g = total + k;
                for (int b2 = b1 + 1; b2 < a.npbc; ++b2) {
                    if (!sd[b2]) continue;
                    a.gorig[g] = n;
                    a.pkey[P + g] = a.pkey[n];
                    for (int q = 0; q < 3; ++q) {
                        const double v1 = sd[b1] > 0 ? a.pv[b1][q] : -1.0 * a.pv[b1][q];
                        const double v2 = sd[b2] > 0 ? a.pv[b2][q] : -1.0 * a.pv[b2][q];
                        a.gvec[(long long)q * a.gcap + g] = v1 + v2;
                    }
                    a.comp[6 * n + a.ccnt[n]++] = P + g;
                    ++g;
                }
            }
            total += sum;
        }
    }
    __syncthreads();
    for (int g = threadIdx.x; g < total; g += blockDim.x) {  // ghostUpdate (elmt.cpp:292-299)
        const int o = a.gorig[g];
        for (int q = 0; q < 3; ++q) a.px[q * st + P + g] = a.px[q * st + o] + a.gvec[(long long)q * a.gcap + g];
    }
    for (int e = threadIdx.x; e < E; e += blockDim.x) {  // the element's ghosts, ascending index
        int* l = a.ecomp + 6 * (long long)a.efirst[e];
        int n = 0;
        for (int p = a.efirst[e]; p < a.efirst[e + 1]; ++p)
            for (int k = 0; k < a.ccnt[p]; ++k) {
                const int v = a.comp[6 * p + k];
                int m = n - 1;
                while (m >= 0 && l[m] > v) { l[m + 1] = l[m]; --m; }
                l[m + 1] = v;
                ++n;
            }
        a.eccnt[e] = n;
    }
    if (threadIdx.x == 0) {
        a.gmeta[0] = total;
        a.gmeta[1] = a.npbc > 0;  // newNeighborList (DEM.cpp:1396-1411): the lattice re-marks its particle nodes
    }
    __syncthreads();
}

__device__ __forceinline__ void nbr_push(const DemArgs& a, int i, int j) {
    const int k = atomicAdd(a.nbr_cnt + i, 1);
    if (k < a.nbr_cap) a.nbr[(long long)i * a.nbr_cap + k] = j;
}

// The reference's sweep (DEM.cpp:1425-1479) from particle p's cell: the 14 half-shell
// offsets, an index that reaches nCells wrapping to 0 and one below 0 taken as the
// unsigned value it becomes there, p paired with every particle of the target cell (with
// a lower index in its own cell) of another element within nebrRange.  Each pair is
// pushed into the candidate list of each of its standard particles.
__device__ __noinline__ void nl_pairs_pbc(const DemArgs& a, int p) {
    constexpr int SH[14][3] = {{0, 0, 0}, {1, 0, 0},  {1, 1, 0},  {0, 1, 0},   {-1, 1, 0}, {0, 0, 1},  {1, 0, 1},
                               {1, 1, 1}, {0, 1, 1}, {-1, 1, 1}, {-1, 0, 1}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1}};
    const int P = a.P;
    const long long st = (long long)P + a.gcap;
    const int c = a.cell_of[p];
    if (c < 0) return;
    const int ep = a.pkey[p];
    const V xp{a.px[p], a.px[st + p], a.px[2 * st + p]};
    const double r2 = a.nebrRange * a.nebrRange;
    const unsigned n0 = (unsigned)a.nC0, n1 = (unsigned)a.nC1, n2 = (unsigned)a.nC2;
    const int i0[3] = {c % a.nC0, (c / a.nC0) % a.nC1, c / (a.nC0 * a.nC1)};
    const unsigned nc[3] = {n0, n1, n2};
    for (int s = 0; s < 14; ++s) {
        unsigned i1[3];
        for (int k = 0; k < 3; ++k) {
            i1[k] = (unsigned)(i0[k] + SH[s][k]);
            if (i1[k] == nc[k]) i1[k] = 0u;
        }
        const unsigned cell1 = (i1[2] * n1 + i1[1]) * n0 + i1[0];
        if (cell1 >= (unsigned)a.ncells) continue;  // not reached for three or more cells per axis
        for (int k = a.cell_start[cell1]; k < a.cell_start[cell1 + 1]; ++k) {
            const int q = a.cell_items[k];
            if (s == 0 && !(q < p)) continue;
            if (a.pkey[q] == ep) continue;  // the same element (cluster)
            const V d = sub(V{a.px[q], a.px[st + q], a.px[2 * st + q]}, xp);
            if (!(nrm2(d) < r2)) continue;
            if (p < P) nbr_push(a, p, q);
            if (q < P) nbr_push(a, q, p);
        }
    }
}

// a standard particle's list in ascending order (the pushes come in any order)
__device__ __noinline__ void nl_sort_one(const DemArgs& a, int i) {
    int cnt = a.nbr_cnt[i];
    if (cnt > a.nbr_cap) { atomicOr(a.status + 2, 1); cnt = a.nbr_cap; a.nbr_cnt[i] = cnt; }
    int* l = a.nbr + (long long)i * a.nbr_cap;
    for (int k = 1; k < cnt; ++k) {
        const int v = l[k];
        int m = k - 1;
        while (m >= 0 && l[m] > v) { l[m + 1] = l[m]; --m; }
        l[m + 1] = v;
    }
}

// ---- forces (DEM.cpp:1114-1182, 1801-2136) --------------------------------------------
// Contact forces are rare (a handful of overlapping pairs among ~10^4 candidates), so
// their arithmetic is kept out of line: inlined, it sets the register budget of the whole
// cooperative kernel and makes every phase spill.  Each takes the running sums and
// returns them updated, in the reference's order of operations.
struct FM {
    V f, m;
};

// particleParticleCollision with I = lower index (DEM.cpp:1801-1900), seen by particle i
// slot: the pair's constants (pair_constants), stride apart
__device__ __noinline__ FM pp_contact(const DemArgs& a, int i, int I, int J, V vd, double rI, double rJ, V FP,
                                      V MP, PredBuf pb, const double* slot) {
    const int E = a.E, eI = I, eJ = J;
    const long long st = (long long)a.E * a.nbr_cap;
    const double dist = sqrt(nrm2(vd));
    const double overlap = rI + rJ - dist;
    const V relVel = sub(ld3(pb.x1r, E, eJ), ld3(pb.x1r, E, eI));
    const V en = divs(vd, dist);
    const double vn = dot(relVel, en);
    const V nrv = mul(vn, en);
    const double effMass = slot[0];
    const double effRad = slot[st];
    const bool lin = a.model != HB_HERTZIAN;
    // the linear model's damping coefficients come from the slot (the same expressions)
    const double fn = lin ? fmax(a.kn * overlap + (-slot[2 * st] * vn), 0.0)
                          : normal_contact(a, overlap, vn, effRad, effMass);
    const V nf = mul(fn, en);
    const V vrI = mul(rI, en), vrJ = mul(-rJ, en);
    const V rvc = add(sub(relVel, cross(ld3(pb.wGr, E, eI), vrI)), cross(ld3(pb.wGr, E, eJ), vrJ));
    const V tang = sub(rvc, nrv);
    const double nt = sqrt(nrm2(tang));
    V tf{0, 0, 0};
    const bool hasT = nt != 0.0;
    if (hasT) {
        const double ft = lin ? fmin(slot[3 * st] * nt, a.muPart * fn)
                              : tangential_contact(a, nt, fn, effRad, effMass, a.muPart);
        tf = mul(ft, divs(tang, nt));
    }
    if (i == I) {
        FP = sub(FP, nf);
        if (hasT) { MP = add(MP, cross(vrI, tf)); FP = add(FP, tf); }
    } else {
        FP = add(FP, nf);
        if (hasT) { MP = sub(MP, cross(vrJ, tf)); FP = sub(FP, tf); }
    }
    return FM{FP, MP};
}

// Contact record for the reaction on the wall or object (its FParticle): the normal force
// it loses and the tangential force it gains, in the order the reference applies them.
// flag 0: no contact, 1: normal force only, 2: normal and tangential.
__device__ __forceinline__ void put_rec(double* rec, double flag, V nf, V tf) {
    rec[0] = flag;
    rec[1] = nf.x; rec[2] = nf.y; rec[3] = nf.z;
    rec[4] = tf.x; rec[5] = tf.y; rec[6] = tf.z;
}

// wallParticleCollision (DEM.cpp:1902-1982), static walls, effective overlap 2x
// rvJ: particle centre - element centre (predicted); clu: the element has several
// spheres (its normal force then has a moment, DEM.cpp:1927-1940)
__device__ __noinline__ FM wall_contact(const DemArgs& a, V wn, double overlap, V xpv, V wpg, double ri, double mi,
                                        V FW, V MW, double* rec, V rvJ = V{0, 0, 0}, bool clu = false) {
    const V relVel = sub(xpv, V{0, 0, 0});
    const double vn = dot(relVel, wn);
    const V nrv = mul(vn, wn);
    const double fn = normal_contact(a, 2.0 * overlap, vn, ri, mi);
    const V nf = mul(fn, wn);
    const V vrJ = mul(-ri, wn);
    const V cJ = clu ? add(vrJ, rvJ) : vrJ;
    FW = add(FW, nf);
    if (clu) MW = add(MW, cross(cJ, nf));
    const V tang = sub(add(relVel, cross(wpg, vrJ)), nrv);
    const double nt = sqrt(nrm2(tang));
    V tfw{0, 0, 0};
    if (nt != 0.0) {
        const double ft = tangential_contact(a, nt, fn, ri, mi, a.muWall);
        tfw = mul(ft, divs(tang, nt));
        MW = sub(MW, cross(cJ, tfw));
        FW = sub(FW, tfw);
    }
    put_rec(rec, nt != 0.0 ? 2.0 : 1.0, nf, tfw);  // wallI->FParticle (DEM.cpp:1946, 1977)
    return FM{FW, MW};
}

// objectParticleCollision (DEM.cpp:2060-2136), effective overlap 2x, particle friction
__device__ __noinline__ FM object_contact(const DemArgs& a, int o, V vd, double dist, double overlap, V xpv, V wpg,
                                          double ri, double mi, V FW, V MW, double* rec, V rvJ = V{0, 0, 0},
                                          bool clu = false) {
    const V en = mul(1.0 / dist, vd);
    const V relVel = sub(xpv, V{a.ox1[o], a.ox1[a.O + o], a.ox1[2 * a.O + o]});
    const double vn = dot(relVel, en);
    const V nrv = mul(vn, en);
    const double fn = normal_contact(a, 2.0 * overlap, vn, ri, mi);
    const V nf = mul(fn, en);
    const V vrJ = mul(-ri, en);
    const V cJ = add(vrJ, rvJ);
    FW = add(FW, nf);
    if (clu) MW = add(MW, cross(cJ, nf));
    const V tang = sub(add(relVel, cross(wpg, vrJ)), nrv);
    const double nt = sqrt(nrm2(tang));
    V tfo{0, 0, 0};
    if (nt != 0.0) {
        const double ft = tangential_contact(a, nt, fn, ri, mi, a.muPart);
        tfo = mul(ft, divs(tang, nt));
        MW = sub(MW, cross(cJ, tfo));
        FW = sub(FW, tfo);
    }
    put_rec(rec, nt != 0.0 ? 2.0 : 1.0, nf, tfo);  // objectI->FParticle (DEM.cpp:2103, 2132)
    return FM{FW, MW};
}

// cylinderParticleCollision (DEM.cpp:1984-2058): effective overlap 2x, wall friction; the
// contact point moves with the cylinder (cylinder::getSpeed, utils.cpp:106-120)
__device__ __noinline__ FM cylinder_contact(const DemArgs& a, int c, V xpi, double overlap, V xpv, V wpg, double ri,
                                            double mi, V FW, V MW, V rvJ = V{0, 0, 0}, bool clu = false) {
    const V p1{a.cp1[c][0], a.cp1[c][1], a.cp1[c][2]};
    const V nx{a.cnax[c][0], a.cnax[c][1], a.cnax[c][2]};
    // cylinder::vecDist (utils.cpp:69-82)
    const V proj = add(p1, mul(dot(nx, sub(xpi, p1)), nx));
    const V dfa = sub(xpi, proj);
    const V vd = sub(xpi, add(proj, mul(a.cR[c], divs(dfa, sqrt(nrm2(dfa))))));
    const V cp = sub(xpi, vd);
    const V en = divs(vd, ri - overlap);
    V cpv{0, 0, 0};
    if (a.cmov[c]) {
        const V q = add(p1, mul(dot(nx, sub(cp, p1)), nx));
        cpv = cross(V{a.comg[c][0], a.comg[c][1], a.comg[c][2]}, sub(cp, q));
    }
    const V relVel = sub(xpv, cpv);
    const double vn = dot(relVel, en);
    const V nrv = mul(vn, en);
    const double fn = normal_contact(a, 2.0 * overlap, vn, ri, mi);
    const V nf = mul(fn, en);
    const V vrJ = mul(-ri, en);
    const V cJ = add(vrJ, rvJ);  // + (particle centre - element centre), zero for spheres
    FW = add(FW, nf);
    if (clu) MW = add(MW, cross(cJ, nf));
    const V tang = sub(add(relVel, cross(wpg, vrJ)), nrv);
    const double nt = sqrt(nrm2(tang));
    if (nt != 0.0) {
        const double ft = tangential_contact(a, nt, fn, ri, mi, a.muWall);
        const V tfc = mul(ft, divs(tang, nt));
        MW = sub(MW, cross(cJ, tfc));
        FW = sub(FW, tfc);
    }
    return FM{FW, MW};
}

// contacts of element i by its group of eight lanes (c = 0..7 of group grp of the
// warp): the lanes take candidates (and objects) in list order, lane c == 0 the wall and
// cylinder; the sums use a fixed xor-shuffle tree within the group, so the result is
// reproducible and every lane of the group ends with the totals in v (FParticle,
// MParticle, FWall, MWall).  All 32 lanes of the warp call it (on false for a group
// without an element), because the tree shuffles across the whole warp.
// a: the kernel's parameter block; ga: its device-memory copy for the out-of-line calls
__device__ __forceinline__ void forces_group(const DemArgs& a, const DemArgs& ga, int i, bool on, int c, PredBuf pb,
                                             int& ncont, double v[12]) {
    __shared__ unsigned s_cm[256];  // each lane's overlapping candidates (bit t: k = c + 8 t)
    const int E = a.E;
    V FP{0, 0, 0}, MP{0, 0, 0}, FW{0, 0, 0}, MW{0, 0, 0};
    bool contribP = false, contribW = false;  // this lane added a particle / a wall or object force
    // pass 1: the contact test (DEM.cpp:1801-1900) of this lane's candidates k = c, c + 8, ...
    unsigned m = 0u;
    const V xpi = on ? ld3(pb.x0r, E, i) : V{0, 0, 0};
    const int cnt = on ? a.nbr_cnt[i] : 0;
    for (int k = c, t = 0; k < cnt; k += 8, ++t) {
        const int j = a.nbr[(long long)i * a.nbr_cap + k];
        const int I = min(i, j), J = max(i, j);
        const double sig = a.rad[I] + a.rad[J];
        const V vd = sub(ld3(pb.x0r, E, J), ld3(pb.x0r, E, I));
        if (nrm2(vd) < sig * sig) {
            m |= 1u << t;
            if (i < j) ++ncont;
        }
    }
    // pass 2: the group's contacts, numbered by lane and then by candidate, go round-robin
    // over its eight lanes (contact q on lane q mod 8), and the wall and cylinder tests to
    // the lane after the last one: no lane runs a second contact chain while another has
    // none.  Each lane adds its contacts in increasing q.
    int T = 0;  // the group's contacts
    if (__any_sync(0xffffffffu, m != 0u)) {
        __syncwarp();  // the previous group's pass 2 has read s_cm
        s_cm[threadIdx.x] = m;
        int incl = __popc(m);
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d, 8);
            if (c >= d) incl += y;
        }
        T = __shfl_sync(0xffffffffu, incl, 7, 8);
        __syncwarp();
    }
    const unsigned* gm = s_cm + (threadIdx.x & ~7);
    for (int q = c; q < T; q += 8) {
        int L = 0, base = 0;
        for (; L < 7; ++L) {
            const int nl = __popc(gm[L]);
            if (q < base + nl) break;
            base += nl;
        }
        unsigned mm = gm[L];
        for (int r = q - base; r > 0; --r) mm &= mm - 1u;
        const int k = L + 8 * (__ffs(mm) - 1);
        const int j = a.nbr[(long long)i * a.nbr_cap + k];
        const int I = min(i, j), J = max(i, j);
        const double rI = a.rad[I], rJ = a.rad[J];
        const V vd = sub(ld3(pb.x0r, E, J), ld3(pb.x0r, E, I));
        contribP = true;
        const FM r = pp_contact(ga, i, I, J, vd, rI, rJ, FP, MP, pb, a.npc + (long long)i * a.nbr_cap + k);
        FP = r.f;
        MP = r.m;
    }
    if (on) {
        const double ri = a.rad[i], mi = a.m[i];
        const V xpv = ld3(pb.x1r, E, i);
        const V wpg = ld3(pb.wGr, E, i);
        if (c == (T & 7)) {  // wallParticleCollision (DEM.cpp:1902-1982), static walls
            const int w = a.wall_of[i];
            bool hit = false;
            if (w >= 0) {
                const V wn{a.wn[w][0], a.wn[w][1], a.wn[w][2]};
                const double dist = dot(wn, sub(xpi, V{a.wp[w][0], a.wp[w][1], a.wp[w][2]}));
                const double overlap = ri - dist;
                if (overlap > 0.0) {
                    contribW = hit = true;
                    const FM r = wall_contact(ga, wn, overlap, xpv, wpg, ri, mi, FW, MW, a.wrec + 7 * (long long)i);
                    FW = r.f;
                    MW = r.m;
                }
            }
            if (!hit) a.wrec[7 * (long long)i] = 0.0;
            const int cy = a.cyl_of[i];
            if (cy >= 0) {  // cylinderParticelContacts (DEM.cpp:1719-1746)
                const V d = sub(xpi, V{a.cp1[cy][0], a.cp1[cy][1], a.cp1[cy][2]});
                const V nx{a.cnax[cy][0], a.cnax[cy][1], a.cnax[cy][2]};
                const double dist = a.cR[cy] - sqrt(nrm2(sub(mul(dot(d, nx), nx), d)));
                const double overlap = ri - dist;
                if (overlap > 0.0) {
                    contribW = true;
                    const FM r = cylinder_contact(ga, cy, xpi, overlap, xpv, wpg, ri, mi, FW, MW);
                    FW = r.f;
                    MW = r.m;
                }
            }
        }
        const int oc = a.obj_cnt[i];
        for (int k = c; k < oc; k += 8) {  // objectParticleCollision (DEM.cpp:2060-2136)
            const int o = a.obj[(long long)i * OBJ_CAP + k];
            const V vd = sub(xpi, V{a.ox0[o], a.ox0[a.O + o], a.ox0[2 * a.O + o]});
            const double dist = sqrt(nrm2(vd));
            const double overlap = ri + a.orad[o] - dist;
            double* rec = a.orec + 7 * ((long long)i * OBJ_CAP + k);
            if (!(overlap > 0.0)) {
                rec[0] = 0.0;
                continue;
            }
            contribW = true;
            const FM r = object_contact(ga, o, vd, dist, overlap, xpv, wpg, ri, mi, FW, MW, rec);
            FW = r.f;
            MW = r.m;
        }
    }
    // fixed xor-shuffle tree within each group of eight lanes.  Particle forces: skipped
    // when in every group at most the group's first lane holds one (the group's first
    // lane then holds the totals).  Wall, cylinder and object forces: the tree whenever a
    // lane of the warp holds one (sums that start at +0.0 are never -0.0, so the tree's
    // additions of +0.0 leave a single lane's force as it is).
    const unsigned whoP = __ballot_sync(0xffffffffu, contribP);
    const unsigned whoW = __ballot_sync(0xffffffffu, contribW);
    v[0] = FP.x; v[1] = FP.y; v[2] = FP.z; v[3] = MP.x; v[4] = MP.y; v[5] = MP.z;
    v[6] = FW.x; v[7] = FW.y; v[8] = FW.z; v[9] = MW.x; v[10] = MW.y; v[11] = MW.z;
    if (whoP & ~0x01010101u) {
#pragma unroll
        for (int off = 1; off < 8; off <<= 1)
#pragma unroll
            for (int q = 0; q < 6; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
    } else {
#pragma unroll
        for (int q = 0; q < 6; ++q) v[q] = __shfl_sync(0xffffffffu, v[q], threadIdx.x & 24);
    }
    if (whoW) {
#pragma unroll
        for (int off = 1; off < 8; off <<= 1)
#pragma unroll
            for (int q = 6; q < 12; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
    }
    if (on && c == 0) {
        st3(a.FP, E, i, V{v[0], v[1], v[2]});
        st3(a.MP, E, i, V{v[3], v[4], v[5]});
        st3(a.FW, E, i, V{v[6], v[7], v[8]});
        st3(a.MW, E, i, V{v[9], v[10], v[11]});
    }
}

// ---- per-particle path (periodic faces, multi-sphere elements) ---------------------------

__device__ __forceinline__ V pv3(const double* arr, long long st, int q) { return V{arr[q], arr[st + q], arr[2 * st + q]}; }

// predicted state of particle p for this substep (particle::updatePredicted and
// ghostUpdate, elmt.cpp:261-274, 292-299): centre, velocity, radiusVec
__device__ __noinline__ void part_predict(const DemArgs& a, int p) {
    const int E = a.E, P = a.P;
    const long long st = (long long)P + a.gcap;
    const int o = p < P ? p : a.gorig[p - P];
    const int e = a.pkey[o];
    V x = ld3(a.xp0, E, e), v = ld3(a.xp1, E, e), rv{0, 0, 0};
    if (a.esize[e] > 1) {
        const V pr{a.proto[o], a.proto[P + o], a.proto[2 * P + o]};
        x = add(x, mul(a.rad[e], project(pr, ldq(a.qp0, E, e))));
        rv = sub(x, ld3(a.xp0, E, e));
        v = add(v, cross(ld3(a.wpG, E, e), rv));
    }
    if (p >= P) {
        const int g = p - P;
        x = add(x, V{a.gvec[g], a.gvec[a.gcap + g], a.gvec[2 * a.gcap + g]});
    }
    a.ppos[p] = x.x; a.ppos[st + p] = x.y; a.ppos[2 * st + p] = x.z;
    a.pvel[p] = v.x; a.pvel[st + p] = v.y; a.pvel[2 * st + p] = v.z;
    a.prv[p] = rv.x; a.prv[st + p] = rv.y; a.prv[2 * st + p] = rv.z;
}

// particleParticleCollision (DEM.cpp:1801-1900) between particles I < J of elements eI, eJ,
// seen by particle `self` (I or J): particle velocities include the element spin, the
// lever arms include radiusVec, and the normal force has a moment on multi-sphere
// elements.  Only standard particles take forces (a ghost's copy acts on its own side).
__device__ __noinline__ FM pp_contact_gen(const DemArgs& a, bool selfI, int I, int J, int eI, int eJ, V vd, double rI,
                                          double rJ, V FP, V MP) {
    const int E = a.E;
    const long long st = (long long)a.P + a.gcap;
    const double dist = sqrt(nrm2(vd));
    const double overlap = rI + rJ - dist;
    const V relVel = sub(pv3(a.pvel, st, J), pv3(a.pvel, st, I));
    const V en = divs(vd, dist);
    const double vn = dot(relVel, en);
    const V nrv = mul(vn, en);
    const double mI = a.m[eI], mJ = a.m[eJ];
    const double effMass = mI * mJ / (mI + mJ);
    const double effRad = rI * rJ / (rI + rJ);
    const double fn = normal_contact(a, overlap, vn, effRad, effMass);
    const V nf = mul(fn, en);
    const V vrI = mul(rI, en), vrJ = mul(-rJ, en);
    const V cI = add(vrI, pv3(a.prv, st, I)), cJ = add(vrJ, pv3(a.prv, st, J));
    if (selfI) {
        FP = sub(FP, nf);
        if (a.esize[eI] > 1) MP = sub(MP, cross(cI, nf));
    } else {
        FP = add(FP, nf);
        if (a.esize[eJ] > 1) MP = add(MP, cross(cJ, nf));
    }
    const V rvc = add(sub(relVel, cross(ld3(a.wpG, E, eI), vrI)), cross(ld3(a.wpG, E, eJ), vrJ));
    const V tang = sub(rvc, nrv);
    const double nt = sqrt(nrm2(tang));
    if (nt != 0.0) {
        const double ft = tangential_contact(a, nt, fn, effRad, effMass, a.muPart);
        const V tf = mul(ft, divs(tang, nt));
        if (selfI) { MP = add(MP, cross(cI, tf)); FP = add(FP, tf); }
        else { MP = sub(MP, cross(cJ, tf)); FP = sub(FP, tf); }
    }
    return FM{FP, MP};
}

// contacts of standard particle p by one warp (as forces_warp), into the particle's
// partial sums; the element sums them over its particles before Newton
__device__ void forces_gen(const DemArgs& a, const DemArgs& ga, int p, int lane, int& ncont) {
    const int E = a.E, P = a.P;
    const long long st = (long long)P + a.gcap;
    const int e = a.pkey[p];
    const V xpi = pv3(a.ppos, st, p);
    V FP{0, 0, 0}, MP{0, 0, 0}, FW{0, 0, 0}, MW{0, 0, 0};
    bool contrib = false;
    const int cnt = a.nbr_cnt[p];
    for (int k = lane; k < cnt; k += 32) {
        const int j = a.nbr[(long long)p * a.nbr_cap + k];
        const int I = min(p, j), J = max(p, j);
        const int eI = a.pkey[I], eJ = a.pkey[J];
        const double rI = a.rad[eI], rJ = a.rad[eJ];
        const double sig = rI + rJ;
        const V vd = sub(pv3(a.ppos, st, J), pv3(a.ppos, st, I));
        if (!(nrm2(vd) < sig * sig)) continue;
        if (p < j) ++ncont;
        contrib = true;
        const FM r = pp_contact_gen(ga, p == I, I, J, eI, eJ, vd, rI, rJ, FP, MP);
        FP = r.f;
        MP = r.m;
    }
    const double ri = a.rad[e], mi = a.m[e];
    const V xpv = pv3(a.pvel, st, p);
    const V wpg = ld3(a.wpG, E, e);
    const V rv = pv3(a.prv, st, p);
    const bool clu = a.esize[e] > 1;
    const int w = a.wall_of[p];
    if (lane == 0) {
        bool hit = false;
        if (w >= 0) {
            const V wn{a.wn[w][0], a.wn[w][1], a.wn[w][2]};
            const double dist = dot(wn, sub(xpi, V{a.wp[w][0], a.wp[w][1], a.wp[w][2]}));
            const double overlap = ri - dist;
            if (overlap > 0.0) {
                contrib = hit = true;
                const FM r = wall_contact(ga, wn, overlap, xpv, wpg, ri, mi, FW, MW, a.wrec + 7 * (long long)p, rv, clu);
                FW = r.f;
                MW = r.m;
            }
        }
        if (!hit) a.wrec[7 * (long long)p] = 0.0;
        const int cy = a.cyl_of[p];
        if (cy >= 0) {
            const V d = sub(xpi, V{a.cp1[cy][0], a.cp1[cy][1], a.cp1[cy][2]});
            const V nx{a.cnax[cy][0], a.cnax[cy][1], a.cnax[cy][2]};
            const double dist = a.cR[cy] - sqrt(nrm2(sub(mul(dot(d, nx), nx), d)));
            const double overlap = ri - dist;
            if (overlap > 0.0) {
                contrib = true;
                const FM r = cylinder_contact(ga, cy, xpi, overlap, xpv, wpg, ri, mi, FW, MW, rv, clu);
                FW = r.f;
                MW = r.m;
            }
        }
    }
    const int oc = a.obj_cnt[p];
    for (int k = lane; k < oc; k += 32) {
        const int o = a.obj[(long long)p * OBJ_CAP + k];
        const V vd = sub(xpi, V{a.ox0[o], a.ox0[a.O + o], a.ox0[2 * a.O + o]});
        const double dist = sqrt(nrm2(vd));
        const double overlap = ri + a.orad[o] - dist;
        double* rec = a.orec + 7 * ((long long)p * OBJ_CAP + k);
        if (!(overlap > 0.0)) {
            rec[0] = 0.0;
            continue;
        }
        contrib = true;
        const FM r = object_contact(ga, o, vd, dist, overlap, xpv, wpg, ri, mi, FW, MW, rec, rv, clu);
        FW = r.f;
        MW = r.m;
    }
    const unsigned who = __ballot_sync(0xffffffffu, contrib);
    double v[12] = {FP.x, FP.y, FP.z, MP.x, MP.y, MP.z, FW.x, FW.y, FW.z, MW.x, MW.y, MW.z};
    if (who & ~1u) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int c = 0; c < 12; ++c) v[c] += __shfl_xor_sync(0xffffffffu, v[c], off);
    }
    if (lane != 0) return;
#pragma unroll
    for (int c = 0; c < 12; ++c) a.pF[(long long)c * P + p] = v[c];
}

// element sums of the particle partials, particles in order: component c of FParticle,
// MParticle, FWall, MWall (c = 0..11)
__device__ __forceinline__ void gather_one(const DemArgs& a, int e, int c) {
    const int E = a.E, P = a.P;
    const int f = a.efirst[e], l = a.efirst[e + 1];
    double s = a.pF[(long long)c * P + f];
    for (int p = f + 1; p < l; ++p) s += a.pF[(long long)c * P + p];
    double* dst = c < 3 ? a.FP : (c < 6 ? a.MP : (c < 9 ? a.FW : a.MW));
    dst[(long long)(c % 3) * E + e] = s;
}

// Newton (DEM.cpp:1149-1181): accelerations from the forces of this substep
__device__ void newton_one(const DemArgs& a, int i, PredBuf pb) {
    const int E = a.E;
    const double ri = a.rad[i], mi = a.m[i];
    const V xpv = ld3(pb.x1r, E, i);
    const V wpg = ld3(pb.wGr, E, i);
    const double nv = a.numVisc;
    const V FVisc = mul(-6.0 * M_PI * nv * ri, xpv);
    const V MVisc = mul(-8.0 * M_PI * nv * ri * ri * ri, wpg);
    const V x2 = add(divs(add(add(add(FVisc, ld3(a.FH, E, i)), ld3(a.FP, E, i)), ld3(a.FW, E, i)), mi),
                     V{a.demF[0], a.demF[1], a.demF[2]});
    st3(a.x2, E, i, x2);
    const V mom = add(add(add(MVisc, ld3(a.MH, E, i)), ld3(a.MP, E, i)), ld3(a.MW, E, i));
    const Qt qp0 = ldq(a.qp0, E, i);
    const V mBf = project(mom, qadj(qp0));
    const V Iv = ld3(a.I, E, i);
    const V wl = ld3(a.wpL, E, i);
    const V waBf{(mBf.x + (Iv.y - Iv.z) * wl.y * wl.z) / Iv.x, (mBf.y + (Iv.z - Iv.x) * wl.z * wl.x) / Iv.y,
                 (mBf.z + (Iv.x - Iv.y) * wl.x * wl.y) / Iv.z};
    st3(a.w1, E, i, project(waBf, qp0));
    if (a.esize && a.esize[i] > 1) {  // q2 = 0.5 qp0 quatAcc(waBf, qp1) (DEM.cpp:1176-1179, vector.cpp:500-504)
        const Qt q1 = ldq(a.qp1, E, i);
        const double n2 = q1.a * q1.a + q1.b * q1.b + q1.c * q1.c + q1.d * q1.d;
        const Qt r = qmul(qp0, Qt{-2.0 * n2, waBf.x, waBf.y, waBf.z});
        stq(a.q2, E, i, Qt{0.5 * r.a, 0.5 * r.b, 0.5 * r.c, 0.5 * r.d});
    }
}

// The same for one Cartesian component of an identity-orientation element (lane c of
// its six: 0-2 linear, 3-5 angular).  With qp0 = identity both projections return their
// argument, so the arithmetic per component is that of newton_one.
// fa, fb: this component's FParticle and FWall (c < 3) or MParticle and MWall (c >= 3).
// A spin lane reads all three components of the predicted local spin while the other two
// spin lanes of its element may already be overwriting theirs with the next prediction:
// the values enter only the Euler terms (I_y - I_z) w_y w_z, ..., which are exactly zero
// for these elements (a single sphere has three equal principal moments), so the result
// does not depend on which value is read.
__device__ double newton_plain(const DemArgs& a, int i, int c, PredBuf pb, double fa, double fb) {
    // One instruction stream for the position lanes (c < 3) and the spin lanes (c >= 3),
    // with selected operands: an FP64 warp instruction costs the same narrow-pipe time
    // whatever its active lanes, so the two chains are not run one after the other.  Per
    // lane the operations and their order are those of the chain it takes:
    //   position: x1 (-6 pi nv ri) + FH + fa + fb, / m, + demF
    //   spin:     w (-8 pi nv ri ri ri) + MH + fa + fb + (I_a - I_b) w_a w_b, / I_k
    const int E = a.E;
    const bool lin = c < 3;
    const int k = lin ? c : c - 3;
    const long long o = (long long)k * E + i;
    const double ri = a.rad[i];
    const double t1 = (lin ? -6.0 * M_PI : -8.0 * M_PI) * a.numVisc;
    const double t2 = t1 * ri;
    const double t4 = (t2 * ri) * ri;
    const double vel = lin ? pb.x1r[o] : pb.wGr[o];
    const double H = lin ? a.FH[o] : a.MH[o];
    const double num = ((vel * (lin ? t2 : t4) + H) + fa) + fb;
    // Euler term of the spin chain (k: (y, z), (z, x), (x, y))
    const int ka = k == 0 ? 1 : (k == 1 ? 2 : 0), kb = k == 0 ? 2 : (k == 1 ? 0 : 1);
    const double Ia = a.I[(long long)ka * E + i], Ib = a.I[(long long)kb * E + i];
    const double wa = a.wpL[(long long)ka * E + i], wb = a.wpL[(long long)kb * E + i];
    const double eul = num + (Ia - Ib) * wa * wb;
    const double q = (lin ? num : eul) / (lin ? a.m[i] : a.I[o]);
    const double qd = q + a.demF[k];
    return lin ? qd : q;
}

__device__ void predict_one(const DemArgs& a, int i) {  // elmt.cpp:139-177
    const int E = a.E;
    const double* c = a.gc;
    const V x0 = ld3(a.x0, E, i), x1 = ld3(a.x1, E, i), x2 = ld3(a.x2, E, i), x3 = ld3(a.x3, E, i),
            x4 = ld3(a.x4, E, i), x5 = ld3(a.x5, E, i);
    st3(a.xp0, E, i, add(add(add(add(add(x0, mul(c[0], x1)), mul(c[1], x2)), mul(c[2], x3)), mul(c[3], x4)), mul(c[4], x5)));
    st3(a.xp1, E, i, add(add(add(add(x1, mul(c[0], x2)), mul(c[1], x3)), mul(c[2], x4)), mul(c[3], x5)));
    st3(a.xp2, E, i, add(add(add(x2, mul(c[0], x3)), mul(c[1], x4)), mul(c[2], x5)));
    st3(a.xp3, E, i, add(add(x3, mul(c[0], x4)), mul(c[1], x5)));
    st3(a.xp4, E, i, add(x4, mul(c[0], x5)));
    st3(a.xp5, E, i, x5);
    const Qt q0 = ldq(a.q0, E, i), q1 = ldq(a.q1, E, i), q2 = ldq(a.q2, E, i), q3 = ldq(a.q3, E, i),
             q4 = ldq(a.q4, E, i), q5 = ldq(a.q5, E, i);
    Qt qp0 = qaxpy(qaxpy(qaxpy(qaxpy(qaxpy(q0, q1, c[0]), q2, c[1]), q3, c[2]), q4, c[3]), q5, c[4]);
    const double qn = sqrt(qp0.a * qp0.a + qp0.b * qp0.b + qp0.c * qp0.c + qp0.d * qp0.d);
    qp0 = Qt{qp0.a / qn, qp0.b / qn, qp0.c / qn, qp0.d / qn};
    stq(a.qp0, E, i, qp0);
    stq(a.qp1, E, i, qaxpy(qaxpy(qaxpy(qaxpy(q1, q2, c[0]), q3, c[1]), q4, c[2]), q5, c[3]));
    stq(a.qp2, E, i, qaxpy(qaxpy(qaxpy(q2, q3, c[0]), q4, c[1]), q5, c[2]));
    stq(a.qp3, E, i, qaxpy(qaxpy(q3, q4, c[0]), q5, c[1]));
    stq(a.qp4, E, i, qaxpy(q4, q5, c[0]));
    stq(a.qp5, E, i, q5);
    const V w0 = ld3(a.w0, E, i), w1 = ld3(a.w1, E, i), w2 = ld3(a.w2, E, i), w3 = ld3(a.w3, E, i),
            w4 = ld3(a.w4, E, i), w5 = ld3(a.w5, E, i);
    const V wp0 = add(add(add(add(add(w0, mul(c[0], w1)), mul(c[1], w2)), mul(c[2], w3)), mul(c[3], w4)), mul(c[4], w5));
    st3(a.wp0, E, i, wp0);
    st3(a.wp1, E, i, add(add(add(add(w1, mul(c[0], w2)), mul(c[1], w3)), mul(c[2], w4)), mul(c[3], w5)));
    st3(a.wp2, E, i, add(add(add(w2, mul(c[0], w3)), mul(c[1], w4)), mul(c[2], w5)));
    st3(a.wp3, E, i, add(add(w3, mul(c[0], w4)), mul(c[1], w5)));
    st3(a.wp4, E, i, add(w4, mul(c[0], w5)));
    st3(a.wp5, E, i, w5);
    st3(a.wpG, E, i, wp0);
    st3(a.wpL, E, i, project(wp0, qadj(qp0)));
}

// displacement trigger (DEM.cpp:1314-1324, 334-347): block maxima, the last block folds
// them and sets the rebuild flag for the next substep
__device__ void trigger_update(const DemArgs& a, double v2) {
    __shared__ double sh[256];
    __shared__ bool last;
    sh[threadIdx.x] = v2;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.partial[blockIdx.x] = sh[0];
        __threadfence();
        last = atomicAdd(a.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double mx = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) mx = fmax(mx, ((volatile double*)a.partial)[b]);
        double md = a.scal[0] + sqrt(mx) * a.dt;
        double flag = 0.0;
        if (md > a.trigger) { md = 0.0; flag = 1.0; }
        a.scal[0] = md;
        a.scal[1] = flag;
        *a.done = 0u;
    }
}

__device__ double correct_one(const DemArgs& a, int i) {  // elmt.cpp:179-254
    const int E = a.E;
    double v2 = 0.0;
    {
        const double* c1o = a.gc1;
        const double* c2o = a.gc2;
        const V x2 = ld3(a.x2, E, i);
        const V x2c = sub(x2, ld3(a.xp2, E, i));
        const V x0 = add(ld3(a.xp0, E, i), mul(c2o[0], x2c));
        const V x1 = add(ld3(a.xp1, E, i), mul(c2o[1], x2c));
        st3(a.x0, E, i, x0);
        st3(a.x1, E, i, x1);
        st3(a.x3, E, i, add(ld3(a.xp3, E, i), mul(c2o[3], x2c)));
        st3(a.x4, E, i, add(ld3(a.xp4, E, i), mul(c2o[4], x2c)));
        st3(a.x5, E, i, add(ld3(a.xp5, E, i), mul(c2o[5], x2c)));
        const V w1 = ld3(a.w1, E, i);
        const V w1c = sub(w1, ld3(a.wp1, E, i));
        const V w0 = add(ld3(a.wp0, E, i), mul(c1o[0], w1c));
        st3(a.w0, E, i, w0);
        st3(a.w2, E, i, add(ld3(a.wp2, E, i), mul(c1o[2], w1c)));
        st3(a.w3, E, i, add(ld3(a.wp3, E, i), mul(c1o[3], w1c)));
        st3(a.w4, E, i, add(ld3(a.wp4, E, i), mul(c1o[4], w1c)));
        st3(a.w5, E, i, add(ld3(a.wp5, E, i), mul(c1o[5], w1c)));
        const Qt q2 = ldq(a.q2, E, i);
        const Qt qp2 = ldq(a.qp2, E, i);
        const Qt q2c = Qt{q2.a - qp2.a, q2.b - qp2.b, q2.c - qp2.c, q2.d - qp2.d};
        Qt q0 = qaxpy(ldq(a.qp0, E, i), q2c, c2o[0]);
        stq(a.q1, E, i, qaxpy(ldq(a.qp1, E, i), q2c, c2o[1]));
        stq(a.q3, E, i, qaxpy(ldq(a.qp3, E, i), q2c, c2o[3]));
        stq(a.q4, E, i, qaxpy(ldq(a.qp4, E, i), q2c, c2o[4]));
        stq(a.q5, E, i, qaxpy(ldq(a.qp5, E, i), q2c, c2o[5]));
        const double qn = sqrt(q0.a * q0.a + q0.b * q0.b + q0.c * q0.c + q0.d * q0.d);
        q0 = Qt{q0.a / qn, q0.b / qn, q0.c / qn, q0.d / qn};
        stq(a.q0, E, i, q0);
        st3(a.wG, E, i, w0);
        st3(a.wL, E, i, project(w0, qadj(q0)));
        v2 = nrm2(x1);
        float* pq = a.pf + 12 * (size_t)i;
        pq[0] = (float)x0.x; pq[1] = (float)x0.y; pq[2] = (float)x0.z;
        pq[3] = (float)x1.x; pq[4] = (float)x1.y; pq[5] = (float)x1.z;
        pq[6] = (float)w0.x; pq[7] = (float)w0.y; pq[8] = (float)w0.z;
    }
    return v2;
}

// first substep after init: trigger from the initial velocities, then predict
// corrector (elmt.cpp:179-254) followed by the next substep's predictor
// (elmt.cpp:139-177) on registers: every input is loaded before the first store, so the
// element's loads overlap instead of waiting on each other
__device__ __noinline__ double correct_predict_one(const DemArgs& a, int i, PredBuf pb) {
    const int E = a.E;
    const double* c = a.gc;
    const double* c1o = a.gc1;
    const double* c2o = a.gc2;
    newton_one(a, i, pb);
    // loads
    const V x2 = ld3(a.x2, E, i), xp0 = ld3(pb.x0r, E, i), xp1 = ld3(pb.x1r, E, i), xp2 = ld3(a.xp2, E, i),
            xp3 = ld3(a.xp3, E, i), xp4 = ld3(a.xp4, E, i), xp5 = ld3(a.xp5, E, i);
    const V w1 = ld3(a.w1, E, i), wp0 = ld3(a.wp0, E, i), wp1 = ld3(a.wp1, E, i), wp2 = ld3(a.wp2, E, i),
            wp3 = ld3(a.wp3, E, i), wp4 = ld3(a.wp4, E, i), wp5 = ld3(a.wp5, E, i);
    const Qt q2 = ldq(a.q2, E, i), qp0 = ldq(a.qp0, E, i), qp1 = ldq(a.qp1, E, i), qp2 = ldq(a.qp2, E, i),
             qp3 = ldq(a.qp3, E, i), qp4 = ldq(a.qp4, E, i), qp5 = ldq(a.qp5, E, i);
    // corrector
    const V x2c = sub(x2, xp2);
    const V x0 = add(xp0, mul(c2o[0], x2c));
    const V x1 = add(xp1, mul(c2o[1], x2c));
    const V x3 = add(xp3, mul(c2o[3], x2c));
    const V x4 = add(xp4, mul(c2o[4], x2c));
    const V x5 = add(xp5, mul(c2o[5], x2c));
    const V w1c = sub(w1, wp1);
    const V w0 = add(wp0, mul(c1o[0], w1c));
    const V w2 = add(wp2, mul(c1o[2], w1c));
    const V w3 = add(wp3, mul(c1o[3], w1c));
    const V w4 = add(wp4, mul(c1o[4], w1c));
    const V w5 = add(wp5, mul(c1o[5], w1c));
    const Qt q2c = Qt{q2.a - qp2.a, q2.b - qp2.b, q2.c - qp2.c, q2.d - qp2.d};
    Qt q0 = qaxpy(qp0, q2c, c2o[0]);
    const Qt q1 = qaxpy(qp1, q2c, c2o[1]);
    const Qt q3 = qaxpy(qp3, q2c, c2o[3]);
    const Qt q4 = qaxpy(qp4, q2c, c2o[4]);
    const Qt q5 = qaxpy(qp5, q2c, c2o[5]);
    const double qn = sqrt(q0.a * q0.a + q0.b * q0.b + q0.c * q0.c + q0.d * q0.d);
    q0 = Qt{q0.a / qn, q0.b / qn, q0.c / qn, q0.d / qn};
    const V wL = project(w0, qadj(q0));
    // predictor for the next substep
    const V nxp0 = add(add(add(add(add(x0, mul(c[0], x1)), mul(c[1], x2)), mul(c[2], x3)), mul(c[3], x4)), mul(c[4], x5));
    const V nxp1 = add(add(add(add(x1, mul(c[0], x2)), mul(c[1], x3)), mul(c[2], x4)), mul(c[3], x5));
    const V nxp2 = add(add(add(x2, mul(c[0], x3)), mul(c[1], x4)), mul(c[2], x5));
    const V nxp3 = add(add(x3, mul(c[0], x4)), mul(c[1], x5));
    const V nxp4 = add(x4, mul(c[0], x5));
    Qt nqp0 = qaxpy(qaxpy(qaxpy(qaxpy(qaxpy(q0, q1, c[0]), q2, c[1]), q3, c[2]), q4, c[3]), q5, c[4]);
    const double pn = sqrt(nqp0.a * nqp0.a + nqp0.b * nqp0.b + nqp0.c * nqp0.c + nqp0.d * nqp0.d);
    nqp0 = Qt{nqp0.a / pn, nqp0.b / pn, nqp0.c / pn, nqp0.d / pn};
    const Qt nqp1 = qaxpy(qaxpy(qaxpy(qaxpy(q1, q2, c[0]), q3, c[1]), q4, c[2]), q5, c[3]);
    const Qt nqp2 = qaxpy(qaxpy(qaxpy(q2, q3, c[0]), q4, c[1]), q5, c[2]);
    const Qt nqp3 = qaxpy(qaxpy(q3, q4, c[0]), q5, c[1]);
    const Qt nqp4 = qaxpy(q4, q5, c[0]);
    const V nwp0 = add(add(add(add(add(w0, mul(c[0], w1)), mul(c[1], w2)), mul(c[2], w3)), mul(c[3], w4)), mul(c[4], w5));
    const V nwp1 = add(add(add(add(w1, mul(c[0], w2)), mul(c[1], w3)), mul(c[2], w4)), mul(c[3], w5));
    const V nwp2 = add(add(add(w2, mul(c[0], w3)), mul(c[1], w4)), mul(c[2], w5));
    const V nwp3 = add(add(w3, mul(c[0], w4)), mul(c[1], w5));
    const V nwp4 = add(w4, mul(c[0], w5));
    const V nwpL = project(nwp0, qadj(nqp0));
    // stores
    st3(a.x0, E, i, x0); st3(a.x1, E, i, x1); st3(a.x3, E, i, x3); st3(a.x4, E, i, x4); st3(a.x5, E, i, x5);
    st3(a.w0, E, i, w0); st3(a.w2, E, i, w2); st3(a.w3, E, i, w3); st3(a.w4, E, i, w4); st3(a.w5, E, i, w5);
    stq(a.q0, E, i, q0); stq(a.q1, E, i, q1); stq(a.q3, E, i, q3); stq(a.q4, E, i, q4); stq(a.q5, E, i, q5);
    st3(a.wG, E, i, w0);
    st3(a.wL, E, i, wL);
    float* pq = a.pf + 12 * (size_t)i;
    pq[0] = (float)x0.x; pq[1] = (float)x0.y; pq[2] = (float)x0.z;
    pq[3] = (float)x1.x; pq[4] = (float)x1.y; pq[5] = (float)x1.z;
    pq[6] = (float)w0.x; pq[7] = (float)w0.y; pq[8] = (float)w0.z;
    st3(pb.x0w, E, i, nxp0); st3(pb.x1w, E, i, nxp1); st3(a.xp2, E, i, nxp2); st3(a.xp3, E, i, nxp3);
    st3(a.xp4, E, i, nxp4); st3(a.xp5, E, i, x5);
    stq(a.qp0, E, i, nqp0); stq(a.qp1, E, i, nqp1); stq(a.qp2, E, i, nqp2); stq(a.qp3, E, i, nqp3);
    stq(a.qp4, E, i, nqp4); stq(a.qp5, E, i, q5);
    st3(a.wp0, E, i, nwp0); st3(a.wp1, E, i, nwp1); st3(a.wp2, E, i, nwp2); st3(a.wp3, E, i, nwp3);
    st3(a.wp4, E, i, nwp4); st3(a.wp5, E, i, w5);
    st3(pb.wGw, E, i, nwp0);
    st3(a.wpL, E, i, nwpL);
    return nrm2(x1);
}

// Elements whose orientation stays the identity (single spheres with q0 = (1,0,0,0) and
// no quaternion rates: their q2 is never set, elmt.cpp:139-254 keeps q exactly) need no
// quaternion algebra, and the projections to the body frame are the identity; their
// Gear corrector+predictor splits into independent Cartesian components.  Six lanes
// per element: lanes 0-2 take x, y, z of the position chain, lanes 3-5 of the spin
// chain.  Same arithmetic per component as correct_predict_one.
__device__ double correct_predict_plain(const DemArgs& a, int i, int c, double acc, PredBuf pb) {
    // Lanes 0-2 run the position chain (2nd order: the corrected derivative is x2, weights
    // gc2), lanes 3-5 the spin chain (1st order: w1, weights gc1).  Both have the same
    // shape, so one instruction stream with selected arrays and weights serves the whole
    // warp (an FP64 warp instruction costs the same whatever its active lanes); the
    // arithmetic per component is exactly that of each chain.
    const int E = a.E;
    const double* cc = a.gc;
    const bool lin = c < 3;
    const long long o = (long long)(lin ? c : c - 3) * E + i;
    double* const v0a = lin ? a.x0 : a.w0;
    double* const v1a = lin ? a.x1 : a.w1;
    double* const v2a = lin ? a.x2 : a.w2;
    double* const v3a = lin ? a.x3 : a.w3;
    double* const v4a = lin ? a.x4 : a.w4;
    double* const v5a = lin ? a.x5 : a.w5;
    // read and written copies of the predicted position and velocity (the spin chain's
    // predictions are the element's own)
    const double* const n0r = lin ? pb.x0r : a.wp0;
    const double* const n1r = lin ? pb.x1r : a.wp1;
    double* const n0a = lin ? pb.x0w : a.wp0;
    double* const n1a = lin ? pb.x1w : a.wp1;
    double* const n2a = lin ? a.xp2 : a.wp2;
    double* const n3a = lin ? a.xp3 : a.wp3;
    double* const n4a = lin ? a.xp4 : a.wp4;
    double* const n5a = lin ? a.xp5 : a.wp5;
    double co[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) co[k] = lin ? a.gc2[k] : a.gc1[k];
    const double p0 = n0r[o], p1 = n1r[o], p2 = n2a[o], p3 = n3a[o], p4 = n4a[o], p5 = n5a[o];
    const double d = acc - (lin ? p2 : p1);
    double v0 = p0 + d * co[0], v1 = p1 + d * co[1], v2 = p2 + d * co[2], v3 = p3 + d * co[3],
           v4 = p4 + d * co[4], v5 = p5 + d * co[5];
    if (lin) v2 = acc;
    else v1 = acc;
    v0a[o] = v0; v1a[o] = v1; v2a[o] = v2; v3a[o] = v3; v4a[o] = v4; v5a[o] = v5;
    const double n0 = v0 + v1 * cc[0] + v2 * cc[1] + v3 * cc[2] + v4 * cc[3] + v5 * cc[4];
    n0a[o] = n0;
    n1a[o] = v1 + v2 * cc[0] + v3 * cc[1] + v4 * cc[2] + v5 * cc[3];
    n2a[o] = v2 + v3 * cc[0] + v4 * cc[1] + v5 * cc[2];
    n3a[o] = v3 + v4 * cc[0] + v5 * cc[1];
    n4a[o] = v4 + v5 * cc[0];
    n5a[o] = v5;
    const float f0 = (float)v0, f1 = (float)v1;
    if (lin) {
        a.pf[12 * (size_t)i + c] = f0;
        a.pf[12 * (size_t)i + 3 + c] = f1;
        return v1;
    }
    a.wG[o] = v0;
    a.wL[o] = v0;
    pb.wGw[o] = n0;
    a.wpL[o] = n0;
    a.pf[12 * (size_t)i + 6 + (c - 3)] = f0;
    return 0.0;
}

__global__ void __launch_bounds__(256) k_dem_first(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v2 = 0.0;
    if (i < a.E) v2 = nrm2(ld3(a.x1, a.E, i));
    trigger_update(a, v2);
    if (i < a.E) predict_one(a, i);
}

// ---- coupling -----------------------------------------------------------------------
struct CoupleArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    uint8_t* ntype;
    uint32_t* solid;
    const double *x0, *rad;
    int E;
    const void* dv;
    int dv_f64;
    const unsigned long long* hacc;  // fixed-point element sums (FP32/FP16 lattice kernels)
    uint32_t* claim_list;       // [2N] (node, particle) joined in this step
    int* claim_cnt;
    unsigned int* mask_done;    // blocks of the mask kernel that have finished (the last one commits)
    int mbb;                    // moving bounce-back: list the nodes that leave their particle
    uint32_t* pop_list;         // [N] (their populations are refilled before the lattice step)
    int* pop_cnt;
    double* rho;
    struct PartBox* tab;        // [E] spheres of the current step
    const double* mass;
    int free_surface;
    double *FH, *MH, *fvol;
    // per-particle path (periodic faces, multi-sphere elements): P standard particles,
    // ghost g is particle P + g; pkey gives every particle's element
    int ghosts, gcap, P;
    int* gmeta;  // [0] ghosts, [1] re-mark pending
    const int *gorig, *pkey, *efirst, *ecomp, *eccnt;
    const double *gvec, *px, *pcen;
    uint32_t* remark;
    // the body force of the coming lattice step: the mask kernel writes force[] (and its
    // FP32 copy) into lb_force when set_force, so that a cycle graph takes a new force
    // through an update of this kernel node's parameters
    double* lb_force;
    double force[3];
    int set_force;
};

// centre and radius of particle p (the element itself, or on the per-particle path the
// corrected particle centre of this cycle)
__device__ __forceinline__ void part_centre(const CoupleArgs& a, int p, double& cx_, double& cy_, double& cz_,
                                            double& r) {
    const int E = a.E;
    if (!a.ghosts) {
        cx_ = a.x0[p]; cy_ = a.x0[E + p]; cz_ = a.x0[2 * E + p];
        r = a.rad[p];
        return;
    }
    const long long st = (long long)a.P + a.gcap;
    cx_ = a.px[p]; cy_ = a.px[st + p]; cz_ = a.px[2 * st + p];
    r = a.rad[a.pkey[p]];
}

struct Box {
    int x0, y0, z0, nx, ny, nz;
};
__device__ __forceinline__ Box pbox(const CoupleArgs& a, int p, int margin) {
    double cx_, cy_, cz_, r;
    part_centre(a, p, cx_, cy_, cz_, r);
    Box b;
    b.x0 = max(0, (int)floor(cx_ - r) - margin);
    b.y0 = max(0, (int)floor(cy_ - r) - margin);
    b.z0 = max(0, (int)floor(cz_ - r) - margin);
    const int x1 = min(a.X - 1, (int)ceil(cx_ + r) + margin);
    const int y1 = min(a.Y - 1, (int)ceil(cy_ + r) + margin);
    const int z1 = min(a.Z - 1, (int)ceil(cz_ + r) + margin);
    b.nx = max(0, x1 - b.x0 + 1);
    b.ny = max(0, y1 - b.y0 + 1);
    b.nz = max(0, z1 - b.z0 + 1);
    return b;
}
// insideSphere (vector.cpp:153-158) is decided in FP64 with the reference's expression;
// an FP32 screen settles every node whose FP32 distance is farther from the sphere
// surface than a rigorous bound of its own rounding error, because the FP64 pipe of this
// part is narrow.  The centre is kept as integer + fraction, so the screen's error does
// not grow with the lattice size:
//   dx_f = f32(x - ix) - f32(cx - ix): |dx_f - dx| <= u (1 + |dx|),  u = 2^-24,
//   |d2_f - d2| <= 3 u (1 + B)(2B + 1) + 12 u B^2  for |dx|, |dy|, |dz| <= B = 2r,
// and nodes farther than 2r are far outside whatever the rounding.  The window
// [lo, hi] = r^2 -/+ (that bound + 1e-9) is rounded outwards.
struct Sph {
    double cx, cy, cz, r2;
    int ix, iy, iz;
    float fx, fy, fz, lo, hi;
};
__device__ __forceinline__ Sph load_sph(const CoupleArgs& a, int p) {
    Sph s;
    double r;
    part_centre(a, p, s.cx, s.cy, s.cz, r);
    s.r2 = r * r;
    s.ix = (int)floor(s.cx); s.iy = (int)floor(s.cy); s.iz = (int)floor(s.cz);
    s.fx = (float)(s.cx - s.ix); s.fy = (float)(s.cy - s.iy); s.fz = (float)(s.cz - s.iz);
    const double u = 5.9604644775390625e-8, B = 2.0 * r;
    const double M = 3.0 * u * (1.0 + B) * (2.0 * B + 1.0) + 12.0 * u * B * B + 1e-9;
    s.lo = __double2float_rd(s.r2 - M);
    s.hi = __double2float_ru(s.r2 + M);
    return s;
}
// exact int -> float for |v| < 2^22 on the FP32 pipe: the bits of 1.5 * 2^23 + v, minus 1.5 * 2^23
__device__ __forceinline__ float i2f_small(int v) { return __int_as_float(0x4B400000 + v) - 12582912.0f; }

// the FP64 decision, not inlined so that the compiler cannot execute it speculatively
__device__ __noinline__ bool in_sph_exact(const Sph& s, int x, int y, int z) {
    const double dx = x - s.cx, dy = y - s.cy, dz = z - s.cz;
    return dx * dx + dy * dy + dz * dz < s.r2;
}

__device__ __forceinline__ bool in_sph(const Sph& s, int x, int y, int z) {
    const float dxf = i2f_small(x - s.ix) - s.fx, dyf = i2f_small(y - s.iy) - s.fy, dzf = i2f_small(z - s.iz) - s.fz;
    const float d2f = dxf * dxf + dyf * dyf + dzf * dzf;
    if (d2f < s.lo) return true;
    if (d2f > s.hi) return false;
    return in_sph_exact(s, x, y, z);
}

// Sphere of every particle for the current step, built once per particle (FP64 is
// narrow on this part; the mask kernel only reads the table).
struct PartBox {
    Sph s;
};
static_assert(sizeof(PartBox) <= 128, "the context allocates 128 bytes per particle");

__device__ __forceinline__ void build_box(const CoupleArgs& a, int p) { a.tab[p].s = load_sph(a, p); }

// Per-particle path, positions final: particle p's corrected centre (px, for its
// sphere), the centre of its element as the coupling sees it (pcen: the element's
// corrected centre, plus the shift for a ghost -- the lever arm of LB.cpp:1871 is
// node - particle centre + radiusVec) and its FP32 record (that centre, the element's
// velocity and spin) for the reduced-precision lattice kernels.
__device__ __noinline__ void part_state(const DemArgs& a, int p) {
    const int E = a.E, P = a.P;
    const long long st = (long long)P + a.gcap;
    const int o = p < P ? p : a.gorig[p - P];
    const int e = a.pkey[o];
    V x = part_pos_corr(a, o), c = ld3(a.x0, E, e);
    if (p >= P) {
        const int g = p - P;
        const V sh{a.gvec[g], a.gvec[a.gcap + g], a.gvec[2 * a.gcap + g]};
        x = add(x, sh);
        c = add(c, sh);
    }
    a.px[p] = x.x; a.px[st + p] = x.y; a.px[2 * st + p] = x.z;
    a.pcen[p] = c.x; a.pcen[st + p] = c.y; a.pcen[2 * st + p] = c.z;
    float* q = a.pf + 12 * (size_t)p;
    q[0] = (float)c.x; q[1] = (float)c.y; q[2] = (float)c.z;
    for (int k = 0; k < 3; ++k) {
        q[3 + k] = (float)a.x1[(long long)k * E + e];
        q[6 + k] = (float)a.wG[(long long)k * E + e];
    }
}

// findNewActive / findNewSolid test a node against every particle of the element
// (DEM components: the element's own sphere, then its ghosts in creation order,
// LB.cpp:1937-1953, 1984-2001): the first that covers it, or -1
__device__ __forceinline__ int cover_first(const CoupleArgs& a, uint32_t q, int x, int y, int z) {
    if (!a.ghosts) return in_sph(a.tab[q].s, x, y, z) ? (int)q : -1;
    const int e = a.pkey[q];
    for (int p = a.efirst[e]; p < a.efirst[e + 1]; ++p)
        if (in_sph(a.tab[p].s, x, y, z)) return p;
    const int n = a.eccnt[e];
    const int* l = a.ecomp + 6 * (long long)a.efirst[e];
    for (int k = 0; k < n; ++k)
        if (in_sph(a.tab[l[k]].s, x, y, z)) return l[k];
    return -1;
}

// Coupling masks, node-parallel (one thread per lattice node, coalesced):
//  findNewActive (LB.cpp:1921-1967): a particle node no longer covered by its particle
//    leaves it;
//  findNewSolid (LB.cpp:1969-2033): a node that is not a particle node after that and is
//    covered by particle q of one of its 6-linked source nodes m (a particle node that
//    stays) joins q; among several sources the lowest node index m wins, the
//    reference's first-in-particleNodes-order rule (that list is sorted).  Nodes that
//    the reference would add through a source added in the same pass (a displacement
//    above half a lattice unit per step) join in the next step.
// Each node decides only for itself.  A source's own flag may be read before or after
// its own pop; both give the same decision because a source must also still be covered
// (in_sph).  New members are listed and joined after every block has decided (by the
// last block of the mask kernel), so no node added in this
// pass acts as a source in it.
__device__ __forceinline__ void claim_push(const CoupleArgs& a, long long l, unsigned long long best) {
    const int slot = atomicAdd(a.claim_cnt, 1);
    a.claim_list[2 * slot] = (uint32_t)l;
    a.claim_list[2 * slot + 1] = (uint32_t)(best & 0xffffffffu);
}

// moving bounce-back: a node that leaves its particle becomes fluid and is refilled after
// the masks; its density is marked NaN until then, so that the refill of a neighbouring
// node does not average it
__device__ __noinline__ void mbb_pop(const CoupleArgs& a, long long l) {
    a.rho[l] = __longlong_as_double(0x7ff8000000000000LL);
    a.pop_list[atomicAdd(a.pop_cnt, 1)] = (uint32_t)l;
}

// one node with the reference's full link rules (periodic remap, self-linked boundary)
__device__ __noinline__ bool mask_node_general(const CoupleArgs& a, int x, int y, int z) {
    const long long l = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
    const uint8_t t = a.ntype[l];
    bool wrote = false;
    if (t & HB_INSIDE) {
        if (cover_first(a, a.solid[l], x, y, z) >= 0) return false;  // stays
        a.ntype[l] = t & ~HB_INSIDE;                                 // pop
        if (a.mbb) mbb_pop(a, l);
        wrote = true;
    }
    unsigned long long best = ~0ull;
    for (int kk = 1; kk <= 6; ++kk) {  // source m with link d[m][kk] == l
        int mx = x - cx(kk), my = y - cy(kk), mz = z - cz(kk);
        if (mx == 0 && a.per[1]) mx = a.X - 2; else if (mx == a.X - 1 && a.per[0]) mx = 1;
        if (my == 0 && a.per[3]) my = a.Y - 2; else if (my == a.Y - 1 && a.per[2]) my = 1;
        if (mz == 0 && a.per[5]) mz = a.Z - 2; else if (mz == a.Z - 1 && a.per[4]) mz = 1;
        // the reference's link table: interior nodes link arithmetically (with the
        // periodic remap), boundary nodes link to themselves
        if (!(mx > 0 && my > 0 && mz > 0 && mx < a.X - 1 && my < a.Y - 1 && mz < a.Z - 1)) continue;
        const long long m = (long long)mx + (long long)a.X * ((long long)my + (long long)a.Y * mz);
        if (!(a.ntype[m] & HB_INSIDE)) continue;
        int lx = mx + cx(kk), ly = my + cy(kk), lz = mz + cz(kk);
        if (lx == 0 && a.per[0]) lx = a.X - 2; else if (lx == a.X - 1 && a.per[1]) lx = 1;
        if (ly == 0 && a.per[2]) ly = a.Y - 2; else if (ly == a.Y - 1 && a.per[3]) ly = 1;
        if (lz == 0 && a.per[4]) lz = a.Z - 2; else if (lz == a.Z - 1 && a.per[5]) lz = 1;
        if (lx != x || ly != y || lz != z) continue;
        const uint32_t q = a.solid[m];
        if (cover_first(a, q, mx, my, mz) < 0) continue;  // the source itself popped
        const int cq = cover_first(a, q, x, y, z);
        if (cq < 0) continue;
        const unsigned long long key = ((unsigned long long)m << 32) | (uint32_t)cq;
        if (key < best) best = key;
    }
    if (best != ~0ull) claim_push(a, l, best);
    return wrote || best != ~0ull;
}

__device__ __forceinline__ uint8_t byte_of(uint32_t w, int k) { return (uint8_t)(w >> (8 * k)); }

// the claim decision of one node (x, y, z) = l whose 6-neighbour sources in kk order
// (x-1, x+1, y-1, y+1, z-1, z+1) carry the particle flag where bit kk of tm is set: the
// particle q of each flagged source m, the lowest (m, q) among those where q still covers
// m and covers l (findNewSolid, LB.cpp:1969-2033)
__device__ __forceinline__ bool claim_node(const CoupleArgs& a, int x, int y, int z, long long l, unsigned tm) {
    const long long sy = a.X, sz = (long long)a.X * a.Y;
    const long long ms[6] = {l - 1, l + 1, l - sy, l + sy, l - sz, l + sz};
    // the sources' particles in one round of independent loads (own index for
    // non-sources, a valid address); usually every flagged source has the same one
    uint32_t qs[6];
#pragma unroll
    for (int kk = 0; kk < 6; ++kk) qs[kk] = a.solid[((tm >> kk) & 1u) ? ms[kk] : l];
    uint32_t q0 = 0xffffffffu;
    bool several = false;
#pragma unroll
    for (int kk = 0; kk < 6; ++kk)
        if ((tm >> kk) & 1u) {
            if (q0 == 0xffffffffu) q0 = qs[kk];
            else if (qs[kk] != q0) several = true;
        }
    const bool cov0 = in_sph(a.tab[q0].s, x, y, z);
    if (!cov0 && !several) return false;  // just outside its particle: the common case
    unsigned long long best = ~0ull;
#pragma unroll
    for (int kk = 0; kk < 6; ++kk) {
        if (!((tm >> kk) & 1u)) continue;
        const uint32_t q = qs[kk];
        const Sph& sq = a.tab[q].s;
        const bool covered = q == q0 ? cov0 : in_sph(sq, x, y, z);
        if (!covered || !in_sph(sq, x - cx(kk + 1), y - cy(kk + 1), z - cz(kk + 1))) continue;
        const unsigned long long key = ((unsigned long long)ms[kk] << 32) | q;
        if (key < best) best = key;
    }
    if (best != ~0ull) claim_push(a, l, best);
    return best != ~0ull;
}

// The claimed nodes join their particles once every block of the mask pass has decided:
// the last block to finish (a counter of finished blocks, each publishing its pops and
// claims first: a fence by every thread that wrote, then the block barrier) applies the
// list, so no node claimed in the pass acted as a source in it.
__device__ __forceinline__ void commit_when_last(const CoupleArgs& a, bool wrote) {
    __shared__ bool s_last;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthreads = blockDim.x * blockDim.y;
    if (wrote) __threadfence();
    __syncthreads();
    if (tid == 0) {
        const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
        s_last = atomicAdd(a.mask_done, 1u) == nb - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (a.ghosts && tid == 0) a.gmeta[1] = 0;  // re-mark done
    const int n = *(volatile int*)a.claim_cnt;
    for (int q = tid; q < n; q += nthreads) {
        const uint32_t l = a.claim_list[2 * q], p = a.claim_list[2 * q + 1];
        a.ntype[l] = a.ntype[l] | HB_INSIDE;
        a.solid[l] = p;
    }
    if (tid == 0) *a.mask_done = 0u;  // ready for the next pass
}

// Four consecutive nodes of a row per thread, 4-byte loads of the node bytes of the row
// and of the four neighbouring rows, so a thread's loads are in flight together.  A warp
// owns 128 nodes of one row; it first sorts them with ballots into two queues in shared
// memory -- particle nodes (a pop test each) and other nodes with a flagged 6-neighbour (a
// claim test each) -- and then works each queue with all its lanes on the same kind of
// item, instead of each lane walking its own mix of node kinds.  A node that pops joins
// the claim queue when a neighbour carries the flag.  Rows near a periodic face, or of a
// length that is not a multiple of 4, take the general per-node rules.
__global__ void __launch_bounds__(128, 12) k_mask(CoupleArgs a) {
    __shared__ uint32_t s_pop[4][128];    // x | node byte << 16 | neighbour flags << 24
    __shared__ uint32_t s_psk[4][128];    // the particle of a queued particle node
    __shared__ uint32_t s_claim[4][128];  // x | neighbour flags << 16
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x, w = threadIdx.y;
    const unsigned lt = (1u << lane) - 1u;
    const int x0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (a.set_force && (blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y) == 0) {
        a.lb_force[0] = a.force[0]; a.lb_force[1] = a.force[1]; a.lb_force[2] = a.force[2];
        float* ff = reinterpret_cast<float*>(a.lb_force + 3);
        ff[0] = (float)a.force[0]; ff[1] = (float)a.force[1]; ff[2] = (float)a.force[2]; ff[3] = 0.0f;
    }
    const bool valid = x0 < a.X && y < a.Y;
    const bool pnear = ((a.per[0] | a.per[1]) && (x0 < 2 || x0 + 3 > a.X - 3)) ||
                       ((a.per[2] | a.per[3]) && (y < 2 || y > a.Y - 3)) ||
                       ((a.per[4] | a.per[5]) && (z < 2 || z > a.Z - 3));
    const bool general = valid && ((a.X & 3) || pnear || a.ghosts);
    bool wrote = false;  // a pop or a claim of this thread, published before the commit
    if (general)
        for (int k = 0; k < 4 && x0 + k < a.X; ++k) wrote |= mask_node_general(a, x0 + k, y, z);
    const bool fast = valid && !general;
    // without a periodic face nearby every link is plain arithmetic: a source is the
    // interior node one step back, and its forward link lands here
    const long long sy = a.X, sz = (long long)a.X * a.Y;
    const long long l0 = (long long)x0 + sy * y + sz * z;
    const bool iy = y >= 1 && y <= a.Y - 2, iz = z >= 1 && z <= a.Z - 2;
    const uint32_t* w32 = reinterpret_cast<const uint32_t*>(a.ntype);
    uint32_t tw = 0u, wym = 0u, wyp = 0u, wzm = 0u, wzp = 0u;
    uint8_t tl = 0, tr = 0;
    uint32_t sl[4] = {0u, 0u, 0u, 0u};
    if (fast) {
        tw = w32[l0 >> 2];
        wym = (y - 1 >= 1 && iz) ? w32[(l0 - sy) >> 2] : 0u;
        wyp = (y + 1 <= a.Y - 2 && iz) ? w32[(l0 + sy) >> 2] : 0u;
        wzm = (z - 1 >= 1 && iy) ? w32[(l0 - sz) >> 2] : 0u;
        wzp = (z + 1 <= a.Z - 2 && iy) ? w32[(l0 + sz) >> 2] : 0u;
        tl = (x0 - 1 >= 1 && iy && iz) ? a.ntype[l0 - 1] : (uint8_t)0;
        tr = (x0 + 4 <= a.X - 2 && iy && iz) ? a.ntype[l0 + 4] : (uint8_t)0;
        if (tw & 0x10101010u) {  // HB_INSIDE in any of the four bytes
            const uint4 v = *reinterpret_cast<const uint4*>(a.solid + l0);
            sl[0] = v.x; sl[1] = v.y; sl[2] = v.z; sl[3] = v.w;
        }
    }
    // Source flags of the four nodes at once, in kk order (x-1, x+1, y-1, y+1, z-1, z+1):
    // the particle bit (0x10) of every byte of the six neighbour words moved to bits 0-5
    // of the node's byte.  A source along x must be an interior node of an interior row;
    // the y and z sources count for interior nodes x (their words are 0 where the source
    // row is not interior).
    static_assert(HB_INSIDE == 0x10, "the shifts below move bit 4 of each byte");
    const uint32_t IN4 = 0x01010101u * HB_INSIDE;
    uint32_t m0 = 0u, m1 = 0u, mx = 0u;  // 0xFF in the bytes where each kind of source counts
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = x0 + k;
        if (x - 1 >= 1) m0 |= 0xFFu << (8 * k);
        if (x + 1 <= a.X - 2) m1 |= 0xFFu << (8 * k);
        if (x >= 1 && x <= a.X - 2) mx |= 0xFFu << (8 * k);
    }
    const uint32_t wxm = (iy && iz) ? ((tw << 8) | tl) & m0 : 0u;
    const uint32_t wxp = (iy && iz) ? ((tw >> 8) | ((uint32_t)tr << 24)) & m1 : 0u;
    const uint32_t nb = ((wxm & IN4) >> 4) | ((wxp & IN4) >> 3) | ((wym & mx & IN4) >> 2) |
                        ((wyp & mx & IN4) >> 1) | (wzm & mx & IN4) | ((wzp & mx & IN4) << 1);
    // queue the four nodes of every lane (ballots give each item its slot)
    int np = 0, nc = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = x0 + k;
        const uint8_t t = byte_of(tw, k);
        const unsigned bits = (nb >> (8 * k)) & 0x3Fu;
        const bool pc = fast && (t & HB_INSIDE);
        const unsigned bp = __ballot_sync(full, pc);
        if (pc) {
            const int q = np + __popc(bp & lt);
            s_pop[w][q] = (uint32_t)x | ((uint32_t)t << 16) | (bits << 24);
            s_psk[w][q] = k == 0 ? sl[0] : (k == 1 ? sl[1] : (k == 2 ? sl[2] : sl[3]));  // registers
        }
        np += __popc(bp);
        const bool cc = fast && !(t & HB_INSIDE) && bits != 0u;
        const unsigned bc = __ballot_sync(full, cc);
        if (cc) s_claim[w][nc + __popc(bc & lt)] = (uint32_t)x | (bits << 16);
        nc += __popc(bc);
    }
    __syncwarp();
    // findNewActive (LB.cpp:1921-1967): a particle node no longer covered by its particle
    // leaves it; then it may be claimed like any other node
    for (int base = 0; base < np; base += 32) {
        const int q = base + lane;
        bool join = false;
        uint32_t item = 0u;
        if (q < np) {
            item = s_pop[w][q];
            const int x = (int)(item & 0xFFFFu);
            const long long l = l0 - x0 + x;
            if (!in_sph(a.tab[s_psk[w][q]].s, x, y, z)) {
                a.ntype[l] = (uint8_t)((item >> 16) & 0xFFu) & ~HB_INSIDE;  // pop
                if (a.mbb) mbb_pop(a, l);
                join = (item >> 24) != 0u;
                wrote = true;
            }
        }
        const unsigned bj = __ballot_sync(full, join);
        if (join) s_claim[w][nc + __popc(bj & lt)] = (item & 0xFFFFu) | ((item >> 24) << 16);
        nc += __popc(bj);
    }
    __syncwarp();
    // findNewSolid (LB.cpp:1969-2033) on the queued nodes
    for (int q = lane; q < nc; q += 32) {
        const uint32_t item = s_claim[w][q];
        const int x = (int)(item & 0xFFFFu);
        wrote |= claim_node(a, x, y, z, l0 - x0 + x, item >> 16);
    }
    commit_when_last(a, wrote);
}

// element hydrodynamic force, torque and entrained fluid (LB.cpp:1853-1918): fixed
// thread-to-row assignment and a fixed-order tree, so the sum is reproducible
__device__ __noinline__ void reduce_block(const CoupleArgs& a, int p0, double (*sh)[256]) {
    const int E = a.E;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    // the element's particles, then its ghosts (nodes carry the particle that covers
    // them); the lever arm is taken from the element's centre (+ the ghost's shift)
    const int nstd = a.ghosts ? a.efirst[p0 + 1] - a.efirst[p0] : 1;
    const int ncomp = a.ghosts ? nstd + a.eccnt[p0] : 1;
    for (int kc = 0; kc < ncomp; ++kc) {
    const int p = !a.ghosts ? p0 : (kc < nstd ? a.efirst[p0] + kc : a.ecomp[6 * (long long)a.efirst[p0] + kc - nstd]);
    const Box b = pbox(a, p, 1);
    double px, py, pz;
    if (a.ghosts) {
        const long long st = (long long)a.P + a.gcap;
        px = a.pcen[p]; py = a.pcen[st + p]; pz = a.pcen[2 * st + p];
    } else {
        px = a.x0[p]; py = a.x0[E + p]; pz = a.x0[2 * E + p];
    }
    for (int r = threadIdx.x; r < b.ny * b.nz; r += blockDim.x) {
        const int y = b.y0 + r % b.ny, z = b.z0 + r / b.ny;
        const long long base = (long long)a.X * ((long long)y + (long long)a.Y * z);
        for (int xc = b.x0; xc < b.x0 + b.nx; xc += 8) {  // 8 loads in flight per chunk
            uint8_t t8[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) t8[k] = xc + k < b.x0 + b.nx ? a.ntype[base + xc + k] : 0;
            bool in8[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                in8[k] = (t8[k] & HB_INSIDE) && is_active(t8[k]) && a.solid[base + xc + k] == (uint32_t)p;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (!in8[k]) continue;
                const long long i = base + xc + k;
                const int x = xc + k;
                double dvx, dvy, dvz;
                if (a.dv_f64) {
                    const double* d = reinterpret_cast<const double*>(a.dv);
                    dvx = d[i]; dvy = d[a.N + i]; dvz = d[2 * a.N + i];
                } else {
                    const float* d = reinterpret_cast<const float*>(a.dv);
                    dvx = d[i]; dvy = d[a.N + i]; dvz = d[2 * a.N + i];
                }
                const double rx = (x - px) + 0.0, ry = (y - py) + 0.0, rz = (z - pz) + 0.0;
                acc[0] += dvx; acc[1] += dvy; acc[2] += dvz;
                acc[3] += ry * dvz - rz * dvy;
                acc[4] += rz * dvx - rx * dvz;
                acc[5] += rx * dvy - ry * dvx;
                acc[6] += a.free_surface ? a.mass[i] : 1.0;
            }
        }
    }
    }
    __syncthreads();
    for (int c = 0; c < 7; ++c) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int c = 0; c < 7; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.FH[p0] = sh[0][0]; a.FH[E + p0] = sh[1][0]; a.FH[2 * E + p0] = sh[2][0];
        a.MH[p0] = sh[3][0]; a.MH[E + p0] = sh[4][0]; a.MH[2 * E + p0] = sh[5][0];
        a.fvol[p0] = sh[6][0];
    }
}

// the reduced-precision lattice kernels leave the same seven sums as 64-bit fixed-point
// integers; converting them is the whole reduction
__device__ __forceinline__ void convert_sums(const CoupleArgs& a, int p) {
    const int E = a.E;
    double v[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) v[k] = (double)(long long)a.hacc[(long long)k * E + p] * HACC_INV;
    a.FH[p] = v[0]; a.FH[E + p] = v[1]; a.FH[2 * E + p] = v[2];
    a.MH[p] = v[3]; a.MH[E + p] = v[4]; a.MH[2 * E + p] = v[5];
    a.fvol[p] = v[6];
}

__global__ void __launch_bounds__(256) k_couple_reduce(CoupleArgs a) {
    __shared__ double sh[7][256];
    reduce_block(a, blockIdx.x, sh);
}

__global__ void k_convert_sums(CoupleArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < a.E) convert_sums(a, p);
}

// ---- one cooperative kernel per cycle --------------------------------------------------
// phases, separated by grid-wide barriers (the launch is cooperative, so every block is
// resident and the barrier cannot stall):
//   R  hydrodynamic force of every element from the previous lattice step
//   D  multiStep DEM substeps: [neighbour rebuild] forces | correct + next predict +
//      displacement trigger
constexpr size_t GARGS_COUPLE = 2560;  // byte offset of the CoupleArgs copy in the parameter buffer
constexpr size_t GARGS_BYTES = 4608;

struct CycleArgs {
    DemArgs d;
    CoupleArgs c;
    // the same two blocks in device memory, for the out-of-line (rarely taken) paths: a
    // kernel parameter passed by reference to a non-inlined function would be copied to
    // every thread's local memory
    const DemArgs* gd;
    const CoupleArgs* gc;
    int do_reduce, do_dem, do_boxes, multi;
    int bps;                 // resident blocks per SM of this launch (the grid is SMs x bps)
    unsigned long long* ts;  // optional phase timestamps (ns), written by block 0 after each barrier
};

__device__ __forceinline__ void stamp(const CycleArgs& A, int k) {
    if (A.ts && blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        A.ts[k] = t;
    }
}

// Warp-sized tasks (a particle's contacts, a group of five elements' corrector) are laid
// out so that consecutive tasks land on different SMs first and on different warp
// schedulers (warp index mod 4) second: an FP64 warp instruction costs the same narrow-
// pipe time whatever its active lanes, so the schedulers' FP64 pipes, not the lanes, are
// the resource.  With the grid as H blocks per SM slot (S = grid / H): task p runs on
// block (p mod S) + S * h and warp k mod W, where k = (p / S) mod (W * H), h = k / W.
__device__ __forceinline__ void warp_tasks(int& first, int& stride, int H) {
    const int B = gridDim.x, W = blockDim.x >> 5;
    if (H < 1 || B % H) H = 1;
    const int S = B / H;
    const int b = blockIdx.x, w = threadIdx.x >> 5;
    first = (b % S) + S * (w + W * (b / S));
    stride = B * W;
}

// neighbour rebuild with periodic faces (DEM.cpp:1395-1494) by the whole cooperative
// grid, out of line so that its registers do not count against the substep loop
__device__ __noinline__ void rebuild_pbc(const DemArgs* gd, int gt, int gs) {
    cg::grid_group grid = cg::this_grid();
    if (blockIdx.x == 0) {
        ghosts_block(*gd);
        nl_cells_block(*gd);
    }
    grid.sync();
    const int P = gd->P;
    const int S = P + *(volatile int*)gd->gmeta;
    for (int p = gt; p < S; p += gs) nl_pairs_pbc(*gd, p);
    grid.sync();
    for (int i = gt; i < P; i += gs) {
        nl_sort_one(*gd, i);
        nl_near_one(*gd, i);
    }
    grid.sync();  // the contact warps read other threads' candidate lists
}

__device__ __noinline__ void part_boxes(const CoupleArgs* gc, const DemArgs* gd) {
    const int S = gd->P + *(volatile int*)gd->gmeta;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S; p += gridDim.x * blockDim.x) {
        part_state(*gd, p);
        build_box(*gc, p);
    }
}

// every particle's predicted state for the substep (the contacts read other particles')
__device__ __noinline__ void part_predict_all(const DemArgs* gd, int gt, int gs) {
    const int S = gd->P + *(volatile int*)gd->gmeta;
    for (int p = gt; p < S; p += gs) part_predict(*gd, p);
}

// overlapping pairs of the last substep (integer atomics, so the count is exact)
__device__ __forceinline__ void count_contacts(const CycleArgs& A, int s, int ncont) {
    if (s != A.multi - 1) return;
    for (int off = 16; off > 0; off >>= 1) ncont += __shfl_down_sync(0xffffffffu, ncont, off);
    if ((threadIdx.x & 31) == 0 && ncont) {
        atomicAdd(A.d.contacts, ncont);
        atomicAdd(A.d.total_contacts, (unsigned long long)ncont);
    }
}

// PBC: periodic faces with particles (ghost rebuilds); a separate instantiation, so the
// calls of that path cost the other configurations no registers
template <bool PBC>
__global__ void __launch_bounds__(256, PBC ? 2 : 1) k_cycle(CycleArgs A) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[7][256];
    const int E = A.d.E;
    // element loops spread consecutive elements over different blocks, so the FP64 work
    // (narrow pipe on this part) lands on every SM instead of the first few
    const int gt = blockIdx.x + gridDim.x * threadIdx.x;
    const int gs = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    int gw, nw;  // this warp's first task and the task stride (one warp per particle / group)
    warp_tasks(gw, nw, A.bps);
    stamp(A, 0);
    if (A.do_reduce) {
        if (A.c.hacc) {
            for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < E; p += gridDim.x * blockDim.x) convert_sums(A.c, p);
        } else {
            for (int p = blockIdx.x; p < E; p += gridDim.x) reduce_block(*A.gc, p, sh);
        }
    }
    int k = 1;
    if (A.do_dem) {
        double maxDisp = A.d.scal[0];
        bool rebuild = A.d.scal[1] != 0.0;
        // per-substep maxima of |x1|^2 (the last MAX_MULTI slots of the partials array)
        unsigned long long* vmax = reinterpret_cast<unsigned long long*>(A.d.partial + PARTIAL_CAP - MAX_MULTI);
        if (blockIdx.x == 0 && threadIdx.x == 0) *A.d.contacts = 0;
        if (blockIdx.x == 0 && (int)threadIdx.x < A.multi) vmax[threadIdx.x] = 0ull;
        grid.sync();
        stamp(A, k++);
        for (int s = 0; s < A.multi; ++s) {
            if (rebuild) {
                if (PBC) {
                    rebuild_pbc(A.gd, gt, gs);
                } else {
                    if (blockIdx.x == 0) nl_cells_block(*A.gd);
                    grid.sync();
                    for (int i = gt; i < E; i += gs) nl_build_one(*A.gd, i);
                    grid.sync();  // the contact groups read other threads' candidate lists
                }
            }
            stamp(A, k++);
            int ncont = 0;
            double v2 = 0.0;
            if (PBC) {
                // per-particle path: forces into per-particle partials | barrier | element
                // sums, Newton, corrector + predictor in place
                const PredBuf pb = pred_inplace(A.d);
                part_predict_all(A.gd, gt, gs);
                grid.sync();
                for (int p = gw; p < A.d.P; p += nw) forces_gen(A.d, *A.gd, p, lane, ncont);
                count_contacts(A, s, ncont);
                grid.sync();
                const int grp = lane / 6, c = lane - 6 * grp;  // six lanes per element, five per warp
                for (int base = 5 * gw; base < E; base += 5 * nw) {
                    const int i = base + grp;
                    const bool on = grp < 5 && i < E;
                    const bool plain = on && A.d.plain[i];
                    if (on) {  // element sums of its particles' contact forces
                        if (plain) {  // the components lane c's Newton reads
                            gather_one(A.d, i, c);
                            gather_one(A.d, i, 6 + c);
                        } else if (c == 0) {
                            for (int q = 0; q < 12; ++q) gather_one(A.d, i, q);
                        }
                    }
                    double x1c = 0.0;
                    if (plain) {
                        const long long o = (long long)(c % 3) * E + i;
                        const double fa = (c < 3 ? A.d.FP : A.d.MP)[o], fb = (c < 3 ? A.d.FW : A.d.MW)[o];
                        x1c = correct_predict_plain(A.d, i, c, newton_plain(A.d, i, c, pb, fa, fb), pb);
                    } else if (on && c == 0) {
                        v2 = fmax(v2, correct_predict_one(*A.gd, i, pb));
                    }
                    // |x1|^2 in the reference's order (x*x + y*y) + z*z, gathered at lane c = 0
                    const double y1 = __shfl_down_sync(0xffffffffu, x1c, 1);
                    const double z1 = __shfl_down_sync(0xffffffffu, x1c, 2);
                    if (plain && c == 0) v2 = fmax(v2, x1c * x1c + y1 * y1 + z1 * z1);
                }
            } else {
                // single spheres: one group of eight lanes per element does its contacts,
                // Newton, corrector and next predictor with no barrier in between; the
                // predicted position, velocity and spin that contact partners read come
                // from one copy and the prediction goes to the other (alternating by
                // substep), so a group that runs ahead cannot change a partner's inputs
                const PredBuf pb = pred_alternate(A.d, s & 1);
                const int grp = lane >> 3, c = lane & 7;  // eight lanes per element, four per warp
                for (int base = 4 * gw; base < E; base += 4 * nw) {
                    const int i = base + grp;
                    const bool on = i < E;
                    double v[12];
                    forces_group(A.d, *A.gd, i, on, c, pb, ncont, v);
                    const bool plain = on && A.d.plain[i];
                    double x1c = 0.0;
                    if (plain && c < 6) {
                        // this lane's component of FParticle + FWall (c < 3) or of MParticle
                        // + MWall (c >= 3), selected with constant indices
                        double fa = 0.0, fb = 0.0;
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            if (c == q) { fa = v[q]; fb = v[6 + q]; }
                            if (c == 3 + q) { fa = v[3 + q]; fb = v[9 + q]; }
                        }
                        x1c = correct_predict_plain(A.d, i, c, newton_plain(A.d, i, c, pb, fa, fb), pb);
                    } else if (on && !plain && c == 0) {
                        v2 = fmax(v2, correct_predict_one(*A.gd, i, pb));
                    }
                    const double y1 = __shfl_down_sync(0xffffffffu, x1c, 1);
                    const double z1 = __shfl_down_sync(0xffffffffu, x1c, 2);
                    if (plain && c == 0) v2 = fmax(v2, x1c * x1c + y1 * y1 + z1 * z1);
                }
                count_contacts(A, s, ncont);
            }
            // DEM.cpp:1314-1324, 334-347: the largest |x1|^2 of the substep, per warp by
            // shuffles, then one 64-bit atomicMax per warp into this substep's slot
            // (non-negative doubles order like their bit patterns; a maximum does not
            // depend on the order), read back by every thread after the barrier
            unsigned long long vb = (unsigned long long)__double_as_longlong(v2);  // v2 >= 0, never NaN
            for (int off = 16; off > 0; off >>= 1) vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, off));
            if (lane == 0 && vb != 0ull) atomicMax(vmax + s, vb);
            grid.sync();
            stamp(A, k++);
            {
                // one thread per block evaluates the trigger (FP64 square root and compare:
                // narrow-pipe instructions that every warp would otherwise repeat), the
                // block takes it from shared memory; every block gets the same value
                __shared__ double s_md;
                __shared__ int s_rb;
                if (threadIdx.x == 0) {
                    const double mx = __longlong_as_double((long long)((volatile unsigned long long*)vmax)[s]);
                    double md = maxDisp + sqrt(mx) * A.d.dt;
                    const bool rb = md > A.d.trigger;
                    if (rb) md = 0.0;
                    s_md = md;
                    s_rb = rb ? 1 : 0;
                }
                __syncthreads();
                maxDisp = s_md;
                rebuild = s_rb != 0;
            }
        }
        if (!PBC && (A.multi & 1)) {
            // an odd number of substeps leaves the next prediction in the second copy:
            // back into the element arrays, where the next cycle and the downloads read it
            for (int i = gt; i < E; i += gs)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const long long o = (long long)q * E + i;
                    A.d.xp0[o] = A.d.xq0[o];
                    A.d.xp1[o] = A.d.xq1[o];
                    A.d.wpG[o] = A.d.wqG[o];
                }
        }
        if (A.do_boxes) {  // positions are final: boxes for the coupling passes
            if (PBC) part_boxes(A.gc, A.gd);
            else  // spread over the blocks: the sphere table's FP64 work lands on every SM
                for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < E; p += gridDim.x * blockDim.x) build_box(A.c, p);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            A.d.scal[0] = maxDisp;
            A.d.scal[1] = rebuild ? 1.0 : 0.0;
        }
    }
}

// ---- coupling masks: separate full-occupancy kernels, one thread per (particle, row) --
__global__ void __launch_bounds__(256) k_build_boxes(CoupleArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < (a.ghosts ? a.P + a.gmeta[0] : a.E)) build_box(a, p);
}

// per-particle path: particle centres, coupling centres and FP32 records from the
// element state (before k_build_boxes when the cooperative kernel did not build them)
__global__ void __launch_bounds__(256) k_part_state(DemArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < a.P + a.gmeta[0]) part_state(a, p);
}

// updateIndices (LB.cpp:1826-1849) after a neighbour rebuild with periodic faces:
// initializeParticleBoundaries (LB.cpp:475-495) over every particle, ghosts included --
// every node loses its particle flag, and each active node inside a particle takes the
// last such particle in list order (the largest index) -- then resetLists.  Mark pass:
// one block per particle sweeps its box and keeps the largest index + 1 per node.
__global__ void __launch_bounds__(256) k_remark_mark(CoupleArgs a) {
    if (!a.gmeta[1]) return;
    const int S = a.P + a.gmeta[0];
    for (int p = blockIdx.x; p < S; p += gridDim.x) {
        const Box b = pbox(a, p, 1);
        const Sph sp = a.tab[p].s;
        const int n = b.nx * b.ny * b.nz;
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            const int x = b.x0 + r % b.nx, y = b.y0 + (r / b.nx) % b.ny, z = b.z0 + r / (b.nx * b.ny);
            const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
            if (!is_active(a.ntype[i])) continue;
            if (in_sph(sp, x, y, z)) atomicMax(a.remark + i, (uint32_t)p + 1u);
        }
    }
}

// apply pass: every node's flag and particle from the mark pass (particle index of a node
// that ends outside stays as it was, like the reference's solidIndex)
__global__ void __launch_bounds__(256) k_remark_apply(CoupleArgs a) {
    if (!a.gmeta[1]) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x) {
        const uint32_t r = a.remark[i];
        uint8_t t = a.ntype[i] & (uint8_t)~HB_INSIDE;
        if (r) {
            t |= HB_INSIDE;
            a.solid[i] = r - 1u;
            a.remark[i] = 0u;
        }
        a.ntype[i] = t;
    }
}

// the ghosts of the initial positions (DEM.cpp:253-257: the neighbour table built at init)
__global__ void __launch_bounds__(256) k_ghosts_init(DemArgs a) { ghosts_block(a); }


// ---- host side ------------------------------------------------------------------------

static DemArgs dem_args(hb_ctx* c) {
    hb_dem_dev& d = c->d;
    DemArgs a;
    a.E = d.E;
    a.x0 = d.x[0]; a.x1 = d.x[1]; a.x2 = d.x[2]; a.x3 = d.x[3]; a.x4 = d.x[4]; a.x5 = d.x[5];
    a.xp0 = d.xp[0]; a.xp1 = d.xp[1]; a.xp2 = d.xp[2]; a.xp3 = d.xp[3]; a.xp4 = d.xp[4]; a.xp5 = d.xp[5];
    a.w0 = d.w[0]; a.w1 = d.w[1]; a.w2 = d.w[2]; a.w3 = d.w[3]; a.w4 = d.w[4]; a.w5 = d.w[5];
    a.wp0 = d.wp[0]; a.wp1 = d.wp[1]; a.wp2 = d.wp[2]; a.wp3 = d.wp[3]; a.wp4 = d.wp[4]; a.wp5 = d.wp[5];
    a.q0 = d.q[0]; a.q1 = d.q[1]; a.q2 = d.q[2]; a.q3 = d.q[3]; a.q4 = d.q[4]; a.q5 = d.q[5];
    a.qp0 = d.qp[0]; a.qp1 = d.qp[1]; a.qp2 = d.qp[2]; a.qp3 = d.qp[3]; a.qp4 = d.qp[4]; a.qp5 = d.qp[5];
    a.wG = d.wG; a.wL = d.wL; a.wpG = d.wpG; a.wpL = d.wpL;
    a.FH = d.FH; a.MH = d.MH; a.FP = d.FP; a.FW = d.FW; a.MP = d.MP; a.MW = d.MW;
    a.fvol = d.fvol; a.m = d.m; a.I = d.I; a.rad = d.rad;
    a.xq0 = d.alt; a.xq1 = d.alt ? d.alt + 3 * (size_t)d.E : nullptr; a.wqG = d.alt ? d.alt + 6 * (size_t)d.E : nullptr;
    a.pf = d.pf;
    a.plain = d.plain;
    a.cell_of = d.cell_of; a.cell_cnt = d.cell_cnt; a.cell_start = d.cell_start;
    a.cell_fill = d.cell_fill; a.cell_items = d.cell_items;
    a.nbr = d.nbr; a.npc = d.npc; a.nbr_cnt = d.nbr_cnt; a.nbr_cap = d.nbr_cap; a.wall_of = d.wall_of; a.obj = d.obj; a.obj_cnt = d.obj_cnt;
    a.wrec = d.wrec; a.orec = d.orec;
    a.cyl_of = d.cyl_of;
    a.ncyl = (int)std::min<size_t>(c->cyl.size(), DEM_MAX_CYL);
    for (int k = 0; k < DEM_MAX_CYL; ++k) {
        const bool on = k < a.ncyl;
        double nx[3] = {0, 0, 0};
        if (on) {  // cylinder::initAxes (utils.cpp:154-161)
            const double ax[3] = {c->cyl[k].p2[0] - c->cyl[k].p1[0], c->cyl[k].p2[1] - c->cyl[k].p1[1],
                                  c->cyl[k].p2[2] - c->cyl[k].p1[2]};
            const double nrm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
            for (int q = 0; q < 3; ++q) nx[q] = ax[q] / nrm;
        }
        for (int q = 0; q < 3; ++q) {
            a.cp1[k][q] = on ? c->cyl[k].p1[q] : 0.0;
            a.cnax[k][q] = nx[q];
            a.comg[k][q] = on ? c->cyl[k].omega[q] : 0.0;
        }
        a.cR[k] = on ? c->cyl[k].R : 0.0;
        a.cmov[k] = on ? c->cyl[k].moving : 0;
    }
    a.scal = d.scal; a.contacts = d.contacts; a.partial = d.partial; a.done = d.done;
    a.ncells = d.ncells; a.nC0 = d.nCells[0]; a.nC1 = d.nCells[1]; a.nC2 = d.nCells[2];
    a.cw0 = d.cellWidth[0]; a.cw1 = d.cellWidth[1]; a.cw2 = d.cellWidth[2];
    a.nebrRange = d.nebrRange; a.trigger = d.trigger; a.dt = d.dt;
    {
        const double dt = d.dt;
        const double c[5] = {dt, dt * dt / 2.0, dt * dt * dt / 6.0, dt * dt * dt * dt / 24.0, dt * dt * dt * dt * dt / 120.0};
        const double g1[6] = {95.0 / 288.0, 1.0, 25.0 / 24.0, 35.0 / 72.0, 5.0 / 48.0, 1.0 / 120.0};
        const double g2[6] = {3.0 / 16.0, 251.0 / 360.0, 1.0, 11.0 / 18.0, 1.0 / 6.0, 1.0 / 60.0};
        for (int k = 0; k < 5; ++k) a.gc[k] = c[k];
        a.gc1[0] = g1[0] * c[0];
        a.gc2[0] = g2[0] * c[1];
        for (int k = 1; k < 6; ++k) {
            a.gc1[k] = g1[k] * c[0] / c[k - 1];
            a.gc2[k] = g2[k] * c[1] / c[k - 1];
        }
    }
    a.nw = d.nw;
    for (int w = 0; w < MAX_WALLS; ++w)
        for (int k = 0; k < 3; ++k) {
            a.wp[w][k] = d.wall_p[w][k];
            a.wn[w][k] = d.wall_n[w][k];
        }
    a.O = d.O; a.ox0 = d.obj_x0; a.ox1 = d.obj_x1; a.orad = d.obj_r;
    a.model = c->P.contact_model;
    a.kn = c->P.linear_stiff;
    a.damp = d.dampCoeff;
    a.knConst = d.knConst;
    a.ksConst = d.ksConst;
    a.viscTang = c->P.visc_tang;
    a.muPart = c->P.friction_part;
    a.muWall = c->P.friction_wall;
    a.numVisc = c->P.num_visc;
    for (int k = 0; k < 3; ++k) a.demF[k] = c->P.lbF[k];  // DEM.cpp:194
    a.status = c->status;
    a.total_contacts = reinterpret_cast<unsigned long long*>(d.scal + 4);
    a.npbc = d.npbc;
    a.gcap = d.gcap;
    for (int b = 0; b < 3; ++b) {
        const bool on = b < d.npbc;
        const double* v = d.pbc_v[b];
        const double nv = on ? sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) : 1.0;
        for (int q = 0; q < 3; ++q) {  // pbc::setPlanes (utils.cpp:240-245)
            a.pv[b][q] = on ? v[q] : 0.0;
            a.pp1[b][q] = on ? d.pbc_p[b][q] : 0.0;
            a.pp2[b][q] = on ? d.pbc_p[b][q] + v[q] : 0.0;
            a.pn1[b][q] = on ? v[q] / nv : 0.0;
            a.pn2[b][q] = -1.0 * a.pn1[b][q];
        }
    }
    a.gmeta = d.gmeta; a.gorig = d.gorig; a.comp = d.comp; a.ccnt = d.ccnt;
    a.gvec = d.gvec; a.px = d.px;
    a.P = d.gen ? d.P : d.E;
    a.gen = d.gen;
    a.pkey = d.pkey; a.ecomp = d.ecomp; a.eccnt = d.eccnt;
    a.efirst = d.efirst; a.esize = d.esize; a.proto = d.proto;
    a.ppos = d.ppos; a.pvel = d.pvel; a.prv = d.prv; a.pF = d.pF; a.pcen = d.pcen;
    return a;
}

void launch_dem_first_predict(hb_ctx* c) {
    if (c->d.E == 0) return;
    DemArgs a = dem_args(c);
    k_dem_first<<<ceil_div(c->d.E, 256), 256, 0, c->stream>>>(a);
}

static CoupleArgs couple_args(hb_ctx* c) {
    CoupleArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype;
    a.solid = c->solid;
    a.x0 = c->d.x[0];
    a.rad = c->d.rad;
    a.E = c->d.E;
    a.dv = c->dv;
    a.dv_f64 = c->P.precision == HB_FP64;
    a.hacc = c->P.precision == HB_FP64 ? nullptr : c->hacc;
    a.claim_list = c->d.claim_list;
    a.claim_cnt = c->d.claim_cnt;
    a.mask_done = c->d.mask_done;
    a.mbb = c->P.coupling == HB_MOVING_BB ? 1 : 0;
    a.pop_list = c->d.pop_list;
    a.pop_cnt = c->d.pop_cnt;
    a.rho = c->rho;
    a.tab = reinterpret_cast<PartBox*>(c->d.boxes);
    a.mass = c->mass;
    a.free_surface = c->P.free_surface;
    a.FH = c->d.FH; a.MH = c->d.MH; a.fvol = c->d.fvol;
    a.ghosts = c->d.gen;
    a.gcap = c->d.gcap;
    a.P = c->d.gen ? c->d.P : c->d.E;
    a.gmeta = c->d.gmeta; a.gorig = c->d.gorig; a.pkey = c->d.pkey; a.efirst = c->d.efirst;
    a.ecomp = c->d.ecomp; a.eccnt = c->d.eccnt;
    a.gvec = c->d.gvec; a.px = c->d.px; a.pcen = c->d.pcen;
    a.remark = c->d.remark;
    a.lb_force = c->lb_force;
    for (int k = 0; k < 3; ++k) a.force[k] = c->P.lbF[k];
    a.set_force = (c->P.force_field && c->lb_force) ? 1 : 0;
    return a;
}

// the mask kernel's node in a captured cycle graph, or null
cudaGraphNode_t find_mask_node(cudaGraph_t g) {
    size_t n = 0;
    if (!g || cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return nullptr;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return nullptr;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        if (cudaGraphKernelNodeGetParams(nd, &kp) == cudaSuccess && kp.func == reinterpret_cast<void*>(k_mask))
            return nd;
    }
    return nullptr;
}

// the current body force into both cycle graphs: the mask kernel node's captured
// arguments with force[] replaced (launches already enqueued keep theirs)
int update_mask_force(hb_ctx* c) {
    for (int k = 0; k < 2; ++k) {
        cudaKernelNodeParams kp;
        if (cudaGraphKernelNodeGetParams(c->mask_node[k], &kp) != cudaSuccess) return -1;
        CoupleArgs a = *static_cast<const CoupleArgs*>(kp.kernelParams[0]);
        for (int q = 0; q < 3; ++q) a.force[q] = c->P.lbF[q];
        void* args[1] = {&a};
        kp.kernelParams = args;
        kp.extra = nullptr;
        if (cudaGraphExecKernelNodeSetParams(c->gexec[k], c->mask_node[k], &kp) != cudaSuccess) return -1;
    }
    return 0;
}

// per-particle path at init: the particles, the ghosts of the initial positions
// (DEM.cpp:253-257: the neighbour table built at init) and the coupling state
int launch_ghosts_init(hb_ctx* c) {
    if (c->d.E == 0 || !c->d.gen) return 0;
    const DemArgs a = dem_args(c);
    k_ghosts_init<<<1, 256, 0, c->stream>>>(a);
    k_part_state<<<ceil_div(c->d.P + c->d.gcap, 256), 256, 0, c->stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// the device copy of the DEM and coupling parameter blocks (constant after init)
int dem_args_upload(hb_ctx* c) {
    if (c->d.E == 0) return 0;
    static_assert(sizeof(DemArgs) <= GARGS_COUPLE, "DemArgs larger than its slot");
    static_assert(GARGS_COUPLE + sizeof(CoupleArgs) <= GARGS_BYTES, "parameter blocks larger than their buffer");
    if (!c->d.gargs && cudaMalloc(&c->d.gargs, GARGS_BYTES) != cudaSuccess) return -1;
    const DemArgs d = dem_args(c);
    const CoupleArgs cp = couple_args(c);
    if (cudaMemcpy(c->d.gargs, &d, sizeof(d), cudaMemcpyHostToDevice) != cudaSuccess) return -1;
    if (cudaMemcpy(reinterpret_cast<char*>(c->d.gargs) + GARGS_COUPLE, &cp, sizeof(cp), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return -1;
    return 0;
}

// cooperative grid of the instantiation a context runs: every SM times the blocks of 256
// threads that fit on one (resident together, as the grid barrier requires)
static int coop_bps(bool per_particle) {
    static int cached[2] = {0, 0};
    int& b = cached[per_particle ? 1 : 0];
    if (b) return b;
    int occ = 0;
    if (per_particle) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cycle<true>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cycle<false>, 256, 0);
    b = occ < 1 ? 1 : (occ > 4 ? 4 : occ);
    return b;
}

int coop_grid(hb_ctx* c) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int g = sms * coop_bps(c->d.gen != 0);
    if (g > PARTIAL_CAP) g = PARTIAL_CAP;  // one trigger partial per block
    return g;
}

int launch_cycle_coop(hb_ctx* c, int do_reduce, int do_dem, int do_boxes, unsigned long long* ts) {
    if (c->d.E == 0) return 0;
    CycleArgs A;
    A.ts = ts;
    A.d = dem_args(c);
    A.c = couple_args(c);
    A.gd = reinterpret_cast<const DemArgs*>(c->d.gargs);
    A.gc = reinterpret_cast<const CoupleArgs*>(reinterpret_cast<const char*>(c->d.gargs) + GARGS_COUPLE);
    // moving bounce-back in FP64: the force pass after the lattice step wrote the sums
    A.do_reduce = do_reduce && !(c->P.coupling == HB_MOVING_BB && c->P.precision == HB_FP64);
    A.do_dem = do_dem;
    A.do_boxes = do_boxes;
    A.multi = c->d.multi;
    A.bps = coop_bps(c->d.gen != 0);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)coop_grid(c));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (c->d.gen) return cudaLaunchKernelEx(&cfg, k_cycle<true>, A) == cudaSuccess ? 0 : -1;
    return cudaLaunchKernelEx(&cfg, k_cycle<false>, A) == cudaSuccess ? 0 : -1;
}

// findNewActive + findNewSolid (LB.cpp:247-280); boxes come from the cooperative kernel
// when it ran the DEM substeps of this cycle (build == false), else are built here.
// ev (optional, 4 events) brackets the three passes for the phase profiler.
void launch_couple(hb_ctx* c, bool build, int cur, cudaEvent_t* ev) {
    if (c->d.E == 0) return;
    CoupleArgs a = couple_args(c);
    if (build && c->d.gen) k_part_state<<<ceil_div(c->d.P + c->d.gcap, 256), 256, 0, c->stream>>>(dem_args(c));
    if (build) k_build_boxes<<<ceil_div(c->d.P + c->d.gcap, 256), 256, 0, c->stream>>>(a);
    if (a.ghosts && a.remark) {  // after a neighbour rebuild (the kernels return at once otherwise)
        k_remark_mark<<<std::min(c->d.P + c->d.gcap, 152 * 8), 256, 0, c->stream>>>(a);
        k_remark_apply<<<152 * 8, 256, 0, c->stream>>>(a);
    }
    if (ev) cudaEventRecord(ev[0], c->stream);
    cudaMemsetAsync(a.claim_cnt, 0, sizeof(int), c->stream);
    if (a.mbb) cudaMemsetAsync(a.pop_cnt, 0, sizeof(int), c->stream);
    if (ev) cudaEventRecord(ev[1], c->stream);
    k_mask<<<dim3((unsigned)ceil_div(ceil_div(c->X, 4), 32), (unsigned)ceil_div(c->Y, 4), (unsigned)c->Z), dim3(32, 4),
             0, c->stream>>>(a);
    if (ev) cudaEventRecord(ev[2], c->stream);
    if (a.mbb) launch_mbb_nodes(c, cur);
    if (ev) cudaEventRecord(ev[3], c->stream);
}

// Wall and object FParticle (DEM.cpp:1123-1129, 1946, 1977, 2103, 2132): reset at every
// force evaluation, then each contact of the last substep subtracts its normal force and
// adds its tangential force, in the reference's table order (particles in index order,
// objects in index order within a particle).  One thread per wall or object replays the
// records in that order, so the FP64 sums are the reference's own.
__global__ void k_reactions(DemArgs a, double* react) {
    // one warp per wall or object: the lanes scan 32 elements at a time for contacts
    // (rare), then the contacts are added in element order (and slot order within an
    // element) by the whole warp in lockstep
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= a.nw + a.O) return;
    const bool wall = t < a.nw;
    const int o = t - a.nw;
    V F{0, 0, 0};
    for (int base = 0; base < a.P; base += 32) {  // particles (= elements for single spheres)
        const int i = base + lane;
        bool hit = false;
        if (i < a.P) {
            if (wall) {
                hit = a.wall_of[i] == t && a.wrec[7 * (long long)i] != 0.0;
            } else {
                const int oc = a.obj_cnt[i];
                for (int k = 0; k < oc && !hit; ++k)
                    hit = a.obj[(long long)i * OBJ_CAP + k] == o && a.orec[7 * ((long long)i * OBJ_CAP + k)] != 0.0;
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, hit);
        while (m) {
            const int e = base + __ffs(m) - 1;
            m &= m - 1;
            if (wall) {
                const double* r = a.wrec + 7 * (long long)e;
                F = sub(F, V{r[1], r[2], r[3]});
                if (r[0] == 2.0) F = add(F, V{r[4], r[5], r[6]});
            } else {
                const int oc = a.obj_cnt[e];
                for (int k = 0; k < oc; ++k) {
                    if (a.obj[(long long)e * OBJ_CAP + k] != o) continue;
                    const double* r = a.orec + 7 * ((long long)e * OBJ_CAP + k);
                    if (r[0] == 0.0) continue;
                    F = sub(F, V{r[1], r[2], r[3]});
                    if (r[0] == 2.0) F = add(F, V{r[4], r[5], r[6]});
                }
            }
        }
    }
    if (lane != 0) return;
    double* dst = wall ? react + 3 * t : react + 3 * (MAX_WALLS + o);
    dst[0] = F.x; dst[1] = F.y; dst[2] = F.z;
}

void launch_reactions(hb_ctx* c) {
    if (c->d.E == 0 || !c->d.react) return;
    k_reactions<<<ceil_div(c->d.nw + c->d.O, 2), 64, 0, c->stream>>>(dem_args(c), c->d.react);
}

void launch_couple_reduce(hb_ctx* c) {
    if (c->d.E == 0) return;
    CoupleArgs a = couple_args(c);
    if (a.hacc) k_convert_sums<<<ceil_div(c->d.E, 128), 128, 0, c->stream>>>(a);
    else k_couple_reduce<<<c->d.E, 256, 0, c->stream>>>(a);
}

}  // namespace hb
