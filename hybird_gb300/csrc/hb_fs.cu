// hb_fs.cu -- free-surface step (LB::latticeBoltzmannFreeSurfaceStep, LB.cpp:235-245,
// 1492-1804): the mass exchange runs on a compacted list of the interface cells (warp
// ballots over the node byte, one warp per cell), the conversions as full-grid passes
// over the node byte.
//
// The reference walks ordered lists (interface nodes sorted ascending, walked backwards;
// filled/emptied lists; appended new interface cells).  Every conversion rule it applies
// depends only on a node's own state and on neighbour types that the same pass does not
// change, so each rule becomes one parallel pass:
//   K1 mass exchange of interface cells (updateMass)          -> mass2
//   K2 classify: mass > n filled -> fluid, mass < 0 emptied -> gas
//   K3 gas cells next to a filled cell -> interface, initialised from the filled
//      neighbour with the LARGEST index (the reference visits filled cells in descending
//      order and the first visitor initialises the cell), surplus -= 0.01
//   K4 fluid cells next to an emptied cell -> interface, mass = 0.99 n, surplus += 0.01 n
//   K5 mutants (emptied not re-interfaced: surplus += mass; filled not re-interfaced:
//      surplus += mass - n, mass = n) and isolated interface without gas links -> fluid
//   K6 isolated interface without fluid links -> gas (surplus += mass)
//   K7 surplus / count added to every interface cell (redistributeMass)
// The FP64 surplus ledger is summed from per-block partials in a fixed order.  Only the
// summation order of that ledger differs from the reference (rounding level).
//
// Streamed populations: the reference's massStream(j) = f[opp j] - fs[j] needs the
// post-collision value fs[j] of the cell, which the push kernel delivered to the active
// neighbour in direction j (f[j] there), or which a moving wall turned into
// f[opp j] = fs[j] - BBi.  At the very first step fs is the initial equilibrium of the
// cell itself (node::initialize sets f = fs), and the first pass uses that.
#include <algorithm>
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

enum : uint8_t { FS_FILLED = 1, FS_EMPTIED = 2, FS_NEW_A = 4, FS_NEW_B = 8 };
constexpr int FS_PARTS = 4;  // ledger partials: K3, K4, K5, K6
constexpr int FS_BLOCK = 128;  // threads per block along x
constexpr int FS_ZC = 8;       // z planes per block: a thread visits FS_ZC nodes

struct FsArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    uint8_t* ntype;
    void* f;                // current populations (post-streaming)
    double* rho;
    double* u;
    double* hf;
    double* mass;
    double* mass2;
    void* visc;             // persistent viscosity or nullptr
    double init_visc;
    uint8_t* flag;
    double* part;           // [FS_PARTS * blocks]
    int* cnt_part;          // [blocks] interface counts
    double* scal;           // [0] surplus [1] interface count
    const double* force;    // lbF as the free surface sees it (zeroed after the first step
                            // when forceFieldSolve = 0)
    int* first;             // device flag: 1 until the first free-surface step has run
    int* nconv;             // [3] cells filled / emptied by this step's classify; cells whose
                            // activity changed (gas <-> interface) in this step
    int blocks;
    uint32_t* ilist;        // [icap] interface cells at the start of the step (unordered)
    int* icount;            // its length (may exceed icap: the overflow is flagged)
    long long icap;         // capacity of ilist (hb_params.cap_interface, default N)
    int* status;            // device status words (word 2, bit 8: interface list full)
};

// Every pass runs on a 3D grid (x from the thread, y and a group of ZC z planes from the
// block; a thread visits its ZC nodes in turn), so a node's coordinates come without
// divisions.  Light passes take ZC = FS_ZC planes, so block scheduling does not dominate
// them; the mass exchange (18 links of every interface cell) and the redistribution take
// one plane per block, so that a surface lying across the x rows spreads over many
// blocks instead of queueing in one lane.  Neighbours follow the reference's periodic
// remap.
struct Node {
    int x, y, z;
    long long i;
    bool ok;
};
template <int ZC = FS_ZC>
__device__ __forceinline__ Node node_of(const FsArgs& a, int zz) {
    Node n;
    n.x = blockIdx.x * blockDim.x + threadIdx.x;
    n.y = blockIdx.y;
    n.z = blockIdx.z * ZC + zz;
    n.ok = n.x < a.X && n.z < a.Z;
    n.i = (long long)n.x + (long long)a.X * ((long long)n.y + (long long)a.Y * n.z);
    return n;
}
// linear block index of the 3D grid (ledger partial slot)
__device__ __forceinline__ int block_id() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

__device__ __forceinline__ void fs_link3(const FsArgs& a, int x, int y, int z, int j, int& xn, int& yn, int& zn) {
    xn = x + cx(j); yn = y + cy(j); zn = z + cz(j);
    if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
}
__device__ __forceinline__ long long lin(const FsArgs& a, int x, int y, int z) {
    return (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
}
__device__ __forceinline__ long long fs_link(const FsArgs& a, const Node& n, int j) {
    int xn, yn, zn;
    fs_link3(a, n.x, n.y, n.z, j, xn, yn, zn);
    return lin(a, xn, yn, zn);
}
__device__ __forceinline__ bool interior3(const FsArgs& a, int x, int y, int z) {
    return x > 0 && y > 0 && z > 0 && x < a.X - 1 && y < a.Y - 1 && z < a.Z - 1;
}
// the interior cell m with link d[m][opp(k)] == n, if any (the reference's neighbour table:
// interior nodes link arithmetically with the periodic remap, boundary nodes to themselves)
__device__ __forceinline__ bool source_of(const FsArgs& a, const Node& n, int k, long long& m) {
    int xm, ym, zm;
    fs_link3(a, n.x, n.y, n.z, k, xm, ym, zm);
    if (!interior3(a, xm, ym, zm)) return false;
    int xb, yb, zb;
    fs_link3(a, xm, ym, zm, opp(k), xb, yb, zb);
    if (xb != n.x || yb != n.y || zb != n.z) return false;
    m = lin(a, xm, ym, zm);
    return true;
}
__device__ __forceinline__ uint8_t code_of(const FsArgs& a, long long i) { return a.ntype[i] & HB_TYPE_MASK; }

template <class P>
__device__ __forceinline__ double fval(const FsArgs& a, int j, long long i) {
    double v = (double)P::load(reinterpret_cast<const typename P::S*>(a.f) + (long long)j * a.N + i);
    if (P::DEV) v += wgt(j);
    return v;
}

// block-sum of one FP64 value into part[k*blocks + block] (fixed-order tree)
__device__ void block_ledger(const FsArgs& a, int k, double v) {
    __shared__ double sh[FS_BLOCK];
    // most blocks convert nothing: their partial is 0 without FP64 work (narrow pipe)
    if (!__syncthreads_or(__double_as_longlong(v) != 0)) {
        if (threadIdx.x == 0) a.part[(long long)k * a.blocks + block_id()] = 0.0;
        return;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[(long long)k * a.blocks + block_id()] = sh[0];
    __syncthreads();
}

// K1 updateMass (LB.cpp:1492-1590): newMass = mass + sum_j a_j (f[opp j] - fs[j])
// Interface cells at the start of the step, compacted with warp ballots (order within
// the list is irrelevant: each cell's mass exchange is independent of the others).
__global__ void __launch_bounds__(FS_BLOCK) k_fs_ilist(FsArgs a) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int zz = 0; zz < FS_ZC; ++zz) {
        const Node nd = node_of(a, zz);
        const bool is_if = nd.ok && code_of(a, nd.i) == HB_T_INTERFACE;
        const unsigned b = __ballot_sync(full, is_if);
        if (!b) continue;
        int base = 0;
        if (lane == 0) {
            base = atomicAdd(a.icount, __popc(b));
            if (base + __popc(b) > a.icap) atomicOr(a.status + 2, 8);  // the list is full
        }
        base = __shfl_sync(full, base, 0);
        const long long k = (long long)base + __popc(b & ((1u << lane) - 1u));
        if (is_if && k < a.icap) a.ilist[k] = (uint32_t)nd.i;
    }
}

// K1 on the list: one thread per interface cell, its 18 links in order; the sum runs in
// link order, as updateMass adds its terms, so each cell's new mass is the reference's
// expression.  (One cell per thread rather than one per warp: the FP64 work of a cell
// then shares its warp instructions with 31 other cells on this part's narrow FP64 pipe.)
template <class P>
__global__ void __launch_bounds__(256) k_fs_mass_list(FsArgs a) {
    const int n = (int)min((long long)*a.icount, a.icap);
    const bool first = *a.first != 0;
    const uint32_t X = (uint32_t)a.X, XY = (uint32_t)a.X * (uint32_t)a.Y;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x) {
        const uint32_t iu = a.ilist[w];  // node indices fit 32 bits (the list is uint32)
        Node nd;
        nd.x = (int)(iu % X);
        nd.y = (int)((iu % XY) / X);
        nd.z = (int)(iu / XY);
        nd.i = (long long)iu;
        nd.ok = true;
        const long long i = nd.i;
        const double mi = a.mass[i];
        double dm = 0.0;
#pragma unroll
        for (int j = 1; j < Q; ++j) {
            const long long l = fs_link(a, nd, j);
            const uint8_t t = code_of(a, l);
            double av = 0.0;
            if (t == HB_T_INTERFACE) av = 0.5 * (a.mass[l] + mi);
            else if (t == HB_T_FLUID) av = 1.0;
            else if (t == HB_T_DYNWALL) av = 1.0 * mi;  // gas, static walls: averageMass 0
            if (av == 0.0) continue;
            double diff;
            if (t == HB_T_DYNWALL) {  // f[opp j] = fs[j] - BBi: the difference is -BBi
                const double fin = fval<P>(a, opp(j), i);
                const double uw = a.u[l] * cx(j) + a.u[a.N + l] * cy(j) + a.u[2 * a.N + l] * cz(j);
                const double fs = first ? fval<P>(a, j, i) : fin + 6.0 * a.rho[i] * wgt(j) * uw;
                diff = fin - fs;
            } else {
                const long long src = first ? i : l;  // fs[j]: f = fs = f_eq at initialisation,
                                                       // else pushed to the active neighbour
                if (P::DEV) {  // deviations: their FP32 difference is that of the populations
                    using S = typename P::S;
                    const S* fp = reinterpret_cast<const S*>(a.f);
                    const float d = P::load(fp + (long long)opp(j) * a.N + i) - P::load(fp + (long long)j * a.N + src);
                    diff = (double)d;
                } else {
                    diff = fval<P>(a, opp(j), i) - fval<P>(a, j, src);
                }
            }
            dm += 1.0 * av * diff;
        }
        a.mass2[i] = mi + dm;
    }
}

// K2 findInterfaceMutants (LB.cpp:1620-1650)
__device__ __forceinline__ void fs_classify_node(const FsArgs& a, const Node& nd) {
    const long long i = nd.i;
    const uint8_t t = a.ntype[i];
    uint8_t fl = 0;
    if ((t & HB_TYPE_MASK) == HB_T_FLUID) a.mass[i] = a.rho[i];  // fluid mass = n (LB.cpp:1582-1585)
    if ((t & HB_TYPE_MASK) == HB_T_INTERFACE) {
        const double m = a.mass2[i];
        a.mass[i] = m;
        if (m > a.rho[i]) {
            fl = FS_FILLED;
            a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_FLUID;
            atomicAdd(a.nconv, 1);
        } else if (m < 0.0) {
            fl = FS_EMPTIED;
            a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_GAS;
            atomicAdd(a.nconv + 1, 1);
            atomicAdd(a.nconv + 2, 1);
        }
    }
    a.flag[i] = fl;
}
__global__ void __launch_bounds__(FS_BLOCK) k_fs_classify(FsArgs a) {
    for (int zz = 0; zz < FS_ZC; ++zz) {
        const Node nd = node_of(a, zz);
        if (nd.ok) fs_classify_node(a, nd);
    }
}

// K3 smoothenInterface, gas neighbours of filled cells (LB.cpp:1657-1677)
template <class P>
__global__ void __launch_bounds__(FS_BLOCK) k_fs_new_from_filled(FsArgs a) {
    double contrib = 0.0;
    // nothing filled in this step (the usual case): no cell changes, the partial is 0
    if (a.nconv[0] != 0)
    for (int zz = 0; zz < FS_ZC; ++zz) {
    const Node nd = node_of(a, zz);
    const long long i = nd.i;
    if (nd.ok && code_of(a, i) == HB_T_GAS && interior3(a, nd.x, nd.y, nd.z)) {
        long long parent = -1;
        for (int k = 1; k < Q; ++k) {  // filled cell m with link d[m][opp k] == i
            long long m;
            if (!source_of(a, nd, k, m) || !(a.flag[m] & FS_FILLED)) continue;
            if (m > parent) parent = m;
        }
        if (parent >= 0) {
            const long long p = parent;
            const double F[3] = {a.hf[p] + a.force[0], a.hf[a.N + p] + a.force[1], a.hf[2 * a.N + p] + a.force[2]};
            const double ux = 1.0 * F[0] / 2.0 / 1.0 + a.u[p];  // node::initialize, node.cpp:26-38
            const double uy = 1.0 * F[1] / 2.0 / 1.0 + a.u[a.N + p];
            const double uz = 1.0 * F[2] / 2.0 / 1.0 + a.u[2 * a.N + p];
            const double usq = ux * ux + uy * uy + uz * uz;
            using S = typename P::S;
            S* f = reinterpret_cast<S*>(a.f);
            for (int j = 0; j < Q; ++j) {
                const double vu = ux * cx(j) + uy * cy(j) + uz * cz(j);
                double fe = wgt(j) * 1.0 * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
                if (P::DEV) fe -= wgt(j);
                P::store(f + (long long)j * a.N + i, (typename P::T)fe);
            }
            a.rho[i] = 1.0;
            a.u[i] = ux; a.u[a.N + i] = uy; a.u[2 * a.N + i] = uz;
            a.hf[i] = 0.0; a.hf[a.N + i] = 0.0; a.hf[2 * a.N + i] = 0.0;
            a.mass[i] = 0.01 * 1.0;
            if (a.visc) {
                if (P::DEV) reinterpret_cast<float*>(a.visc)[i] = reinterpret_cast<float*>(a.visc)[p];
                else reinterpret_cast<double*>(a.visc)[i] = reinterpret_cast<double*>(a.visc)[p];
            }
            a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_INTERFACE;
            a.flag[i] |= FS_NEW_A;
            atomicAdd(a.nconv + 2, 1);
            contrib += -0.01 * 1.0;
        }
    }
    }
    block_ledger(a, 0, contrib);
}

// K4 smoothenInterface, fluid neighbours of emptied cells (LB.cpp:1679-1700)
__global__ void __launch_bounds__(FS_BLOCK) k_fs_new_from_emptied(FsArgs a) {
    double contrib = 0.0;
    if (a.nconv[1] != 0)
    for (int zz = 0; zz < FS_ZC; ++zz) {
    const Node nd = node_of(a, zz);
    const long long i = nd.i;
    if (nd.ok && code_of(a, i) == HB_T_FLUID && interior3(a, nd.x, nd.y, nd.z)) {
        bool hit = false;
        for (int k = 1; k < Q && !hit; ++k) {
            long long m;
            if (source_of(a, nd, k, m) && (a.flag[m] & FS_EMPTIED)) hit = true;
        }
        if (hit) {
            const double n = a.rho[i];
            a.mass[i] = 0.99 * n;
            contrib += 0.01 * n;
            a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_INTERFACE;
            a.flag[i] |= FS_NEW_B;
        }
    }
    }
    block_ledger(a, 1, contrib);
}

// K5 updateMutants (LB.cpp:1703-1742) and removeIsolated, first pass (LB.cpp:1749-1769)
__global__ void __launch_bounds__(FS_BLOCK) k_fs_mutants_to_fluid(FsArgs a) {
    double contrib = 0.0;
    for (int zz = 0; zz < FS_ZC; ++zz) {
    const Node nd = node_of(a, zz);
    const long long i = nd.i;
    if (nd.ok) {
        const uint8_t fl = a.flag[i];
        const uint8_t t = code_of(a, i);
        if ((fl & FS_EMPTIED) && !(fl & FS_NEW_A)) {
            contrib += a.mass[i];
        } else if ((fl & FS_FILLED) && !(fl & FS_NEW_B)) {
            contrib += a.mass[i] - a.rho[i];
            a.mass[i] = a.rho[i];
        }
        if (t == HB_T_INTERFACE) {
            bool gas = false;
            for (int j = 1; j < Q && !gas; ++j)
                if (code_of(a, fs_link(a, nd, j)) == HB_T_GAS) gas = true;
            if (!gas) {
                contrib += a.mass[i] - a.rho[i];
                a.mass[i] = a.rho[i];
                a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_FLUID;
            }
        }
    }
    }
    block_ledger(a, 2, contrib);
}

// K6 removeIsolated, second pass (LB.cpp:1771-1793)
__global__ void __launch_bounds__(FS_BLOCK) k_fs_isolated_gas(FsArgs a) {
    double contrib = 0.0;
    int count = 0;
    for (int zz = 0; zz < FS_ZC; ++zz) {
    const Node nd = node_of(a, zz);
    const long long i = nd.i;
    if (nd.ok && code_of(a, i) == HB_T_INTERFACE) {
        bool fluid = false;
        for (int j = 1; j < Q && !fluid; ++j)
            if (code_of(a, fs_link(a, nd, j)) == HB_T_FLUID) fluid = true;
        if (!fluid) {
            contrib += a.mass[i];
            a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_GAS;
            atomicAdd(a.nconv + 2, 1);
        } else {
            count += 1;
        }
    }
    }
    block_ledger(a, 3, contrib);
    __shared__ int shc[FS_BLOCK];
    shc[threadIdx.x] = count;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) shc[threadIdx.x] += shc[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.cnt_part[block_id()] = shc[0];
}

// ledger total and interface count: k_fs_ledger_part sums fixed chunks of the block
// partials (one block per chunk, fixed-order tree), k_fs_ledger the chunk sums; zero
// partials are skipped by an integer test of their bits
constexpr int FS_LEDGER_CHUNKS = 256;

__global__ void k_fs_ledger_part(FsArgs a, double* csum, long long* ccnt) {
    __shared__ double shs[256];
    __shared__ long long shc[256];
    const int per = (a.blocks + FS_LEDGER_CHUNKS - 1) / FS_LEDGER_CHUNKS;
    const int b0 = blockIdx.x * per, b1 = min(a.blocks, b0 + per);
    double s = 0.0;
    long long c = 0;
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        for (int k = 0; k < FS_PARTS; ++k) {
            const double v = a.part[(long long)k * a.blocks + b];
            if (__double_as_longlong(v) != 0) s += v;
        }
        c += a.cnt_part[b];
    }
    shs[threadIdx.x] = s;
    shc[threadIdx.x] = c;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            if (__double_as_longlong(shs[threadIdx.x + k]) != 0) shs[threadIdx.x] += shs[threadIdx.x + k];
            shc[threadIdx.x] += shc[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        csum[blockIdx.x] = shs[0];
        ccnt[blockIdx.x] = shc[0];
    }
}

__global__ void k_fs_ledger(FsArgs a, const double* csum, const long long* ccnt) {
    __shared__ double shs[FS_LEDGER_CHUNKS];
    __shared__ long long shc[FS_LEDGER_CHUNKS];
    shs[threadIdx.x] = csum[threadIdx.x];
    shc[threadIdx.x] = ccnt[threadIdx.x];
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            if (__double_as_longlong(shs[threadIdx.x + k]) != 0) shs[threadIdx.x] += shs[threadIdx.x + k];
            shc[threadIdx.x] += shc[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.scal[0] = shs[0];
        a.scal[1] = (double)shc[0];
        *a.first = 0;
        a.nconv[0] = 0;  // counts of the next step's classify
        a.nconv[1] = 0;
    }
}

// K7 redistributeMass (LB.cpp:1796-1804)
__global__ void __launch_bounds__(FS_BLOCK) k_fs_redistribute(FsArgs a) {
    const Node nd = node_of<1>(a, 0);
    if (nd.ok && code_of(a, nd.i) == HB_T_INTERFACE) a.mass[nd.i] += a.scal[0] / a.scal[1];
}

// ---- host side ---------------------------------------------------------------------------

static FsArgs fs_args(hb_ctx* c, int cur) {
    FsArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype;
    a.f = cur ? c->fB : c->fA;
    a.rho = c->rho;
    a.u = c->u;
    a.hf = c->hf;
    a.mass = c->mass;
    a.mass2 = c->fs_mass2;
    a.visc = c->visc;
    a.init_visc = c->P.init_visc;
    a.flag = c->fs_flag;
    a.part = c->fs_part;
    a.cnt_part = c->fs_cnt;
    a.scal = c->fs_scal;
    a.force = c->fs_force;
    a.first = c->fs_first;
    a.nconv = c->fs_first + 1;
    a.blocks = ceil_div(c->X, FS_BLOCK) * c->Y * ceil_div(c->Z, FS_ZC);
    a.ilist = c->fs_ilist;
    a.icount = c->fs_first + 4;
    a.icap = c->fs_icap;
    a.status = c->status;
    return a;
}

void fs_buffer_bytes(const hb_ctx* c, size_t* part, size_t* cnt) {
    const size_t blocks = (size_t)ceil_div(c->X, FS_BLOCK) * c->Y * ceil_div(c->Z, FS_ZC);
    *part = sizeof(double) * (FS_PARTS * blocks + 2 * FS_LEDGER_CHUNKS);
    *cnt = sizeof(int) * blocks;
}

int fs_init(hb_ctx* c) {
    const long long N = c->N;
    const int blocks = ceil_div(c->X, FS_BLOCK) * c->Y * ceil_div(c->Z, FS_ZC);
    if (cudaMalloc(&c->fs_flag, N) != cudaSuccess || cudaMalloc(&c->fs_mass2, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&c->fs_part, sizeof(double) * (FS_PARTS * blocks + 2 * FS_LEDGER_CHUNKS)) != cudaSuccess ||
        cudaMalloc(&c->fs_cnt, sizeof(int) * blocks) != cudaSuccess ||
        cudaMalloc(&c->fs_scal, sizeof(double) * 2) != cudaSuccess ||
        cudaMalloc(&c->fs_first, 6 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&c->fs_ilist, sizeof(uint32_t) * (c->fs_icap = c->P.cap_interface > 0 ? std::min<long long>(c->P.cap_interface, N) : N)) !=
            cudaSuccess)
        return HB_ERR_NOMEM;
    cudaMemset(c->fs_flag, 0, N);
    cudaMemset(c->fs_scal, 0, sizeof(double) * 2);
    const int init[6] = {1, 0, 0, 0, 0, 0};  // first step; filled / emptied / activity-change
                                              // counts; interface-list length
    cudaMemcpy(c->fs_first, init, sizeof(init), cudaMemcpyHostToDevice);
    return cudaGetLastError() == cudaSuccess ? HB_OK : HB_ERR_CUDA;
}

void launch_fs_step(hb_ctx* c, int cur) {
    FsArgs a = fs_args(c, cur);
    const dim3 G((unsigned)ceil_div(c->X, FS_BLOCK), (unsigned)c->Y, (unsigned)ceil_div(c->Z, FS_ZC));
    const dim3 G1((unsigned)ceil_div(c->X, FS_BLOCK), (unsigned)c->Y, (unsigned)c->Z);  // one plane per block
    const int B = FS_BLOCK;
    cudaStream_t s = c->stream;
    cudaMemsetAsync(a.icount, 0, sizeof(int), s);
    k_fs_ilist<<<G, B, 0, s>>>(a);
    const int GL = 152 * 8;  // persistent: 8 blocks of 8 warps per SM over the list
    if (c->P.precision == HB_FP64) k_fs_mass_list<PolF64><<<GL, 256, 0, s>>>(a);
    else if (c->P.precision == HB_FP32) k_fs_mass_list<PolF32><<<GL, 256, 0, s>>>(a);
    else k_fs_mass_list<PolF16><<<GL, 256, 0, s>>>(a);
    k_fs_classify<<<G, B, 0, s>>>(a);
    if (c->P.precision == HB_FP64) k_fs_new_from_filled<PolF64><<<G, B, 0, s>>>(a);
    else if (c->P.precision == HB_FP32) k_fs_new_from_filled<PolF32><<<G, B, 0, s>>>(a);
    else k_fs_new_from_filled<PolF16><<<G, B, 0, s>>>(a);
    k_fs_new_from_emptied<<<G, B, 0, s>>>(a);
    k_fs_mutants_to_fluid<<<G, B, 0, s>>>(a);
    k_fs_isolated_gas<<<G, B, 0, s>>>(a);
    double* csum = reinterpret_cast<double*>(c->fs_part + (size_t)FS_PARTS * a.blocks);
    long long* ccnt = reinterpret_cast<long long*>(csum + FS_LEDGER_CHUNKS);
    k_fs_ledger_part<<<FS_LEDGER_CHUNKS, 256, 0, s>>>(a, csum, ccnt);
    k_fs_ledger<<<1, FS_LEDGER_CHUNKS, 0, s>>>(a, csum, ccnt);
    k_fs_redistribute<<<G1, B, 0, s>>>(a);
    launch_refresh_bulk(c, c->fs_first + 3);  // only when a cell's activity changed
}

}  // namespace hb
