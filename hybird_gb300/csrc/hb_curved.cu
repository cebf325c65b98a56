// hb_curved.cu -- cylinders and curved walls (boundary code 9; LB.cpp:552-603,
// 1278-1319; node.cpp:458-472; utils.cpp:106-120, 177-224).
//
// Every node outside a cylinder becomes a curved wall (LB::initializeCylinderBoundaries
// marks it a wall of the cylinder's kind and then curved).  A population fs[j] that
// leaves active node i toward a curved wall node w comes back as
//   f[opp j] = (1 - chi) fs[j] + chi f*  - BBi,
//   f* = n w_j (1 + 3 c_j.u_bf + 4.5 (c_j.u)^2 + 1.5 u^2),   BBi = 6 n w_j (v_w . c_j)
// with delta = 1 - t, t the distance along c_(opp j) from w to the cylinder surface
// (cylinder::segmentIntercept, as the reference: both roots with the minus sign),
// chi = (2 delta - 1) / tau (delta >= 1/2) or (2 delta - 1) / (tau - 2), and the fluid
// reference velocity u_bf = m1 u + m2 v_w (delta >= 1/2; m1 = (delta - 1) / delta,
// m2 = 1 / delta) or the velocity of the fluid node behind i (else; the wall velocity if
// that node is not fluid).  The 1.5 u^2 term keeps the reference's sign.
//
// The lattice kernels push, so they bounce curved links back unchanged (f_out[opp j][i] =
// fs[j], as a static wall) and write the FP64 velocity of every node the rule reads
// (HB_MIRROR bit); one pass over the static list of (node, curved link) entries then
// applies the rule.  No entry reads a slot another entry writes.  This file is compiled
// without FMA contraction: the FP64 form follows the reference's evaluation order.
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

struct CylDev {
    double p1[3], naxes[3], R, omega[3];
    int moving;
};
constexpr int MAX_CYL = 8;

struct CurvedEntry {
    uint32_t i, back;  // active-capable node, the node behind it along opp(j)
    int j;
    double delta;
    double v[3];       // velocity of the wall node (its node object, LB.cpp:958-990)
};

struct CurvedArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    uint8_t* ntype;
    const uint32_t* solid;
    int ncyl;
    CylDev cyl[MAX_CYL];
    int nw;
    double wp[MAX_WALLS][3], wn[MAX_WALLS][3];
    CurvedEntry* list;
    int* count;
    int cap;
    // step pass
    void* f;
    const double* rho;
    const double* u;
    const void* visc;
    int visc_kind;  // 0 constant, 1 float, 2 double
    double init_visc;
};

__device__ __forceinline__ void pos_of(const CurvedArgs& a, long long i, double* p) {
    p[0] = (double)(i % a.X);
    p[1] = (double)((i / a.X) % a.Y);
    p[2] = (double)(i / ((long long)a.X * a.Y));
}

__device__ __forceinline__ long long link_of(const CurvedArgs& a, long long i, int j) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
    return (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
}
__device__ __forceinline__ bool interior(const CurvedArgs& a, long long i) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    return x > 0 && y > 0 && z > 0 && x < a.X - 1 && y < a.Y - 1 && z < a.Z - 1;
}

// tinyVector::insideCylinder (vector.cpp:160-170)
__device__ __forceinline__ bool inside_cyl(const CylDev& c, const double* p) {
    const double d[3] = {p[0] - c.p1[0], p[1] - c.p1[1], p[2] - c.p1[2]};
    const double s = d[0] * c.naxes[0] + d[1] * c.naxes[1] + d[2] * c.naxes[2];
    const double q[3] = {d[0] - s * c.naxes[0], d[1] - s * c.naxes[1], d[2] - s * c.naxes[2]};
    return q[0] * q[0] + q[1] * q[1] + q[2] * q[2] < c.R * c.R;
}

// LB::initializeCylinderBoundaries (LB.cpp:552-586): nodes outside a cylinder become
// curved walls (after the lattice boundaries, particles and walls; before the objects)
__global__ void k_cyl_types(CurvedArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    double p[3];
    pos_of(a, i, p);
    for (int c = 0; c < a.ncyl; ++c)
        if (!inside_cyl(a.cyl[c], p)) a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_CURVED;
}

// cylinder::segmentIntercept (utils.cpp:177-224): the reference takes the smaller of two
// roots that are both computed with -sqrt, and returns 0 when there is none
__device__ __forceinline__ double segment_intercept(const CylDev& c, const double* start, const double* dir,
                                                    const double* p2) {
    const double AB[3] = {p2[0] - c.p1[0], p2[1] - c.p1[1], p2[2] - c.p1[2]};
    const double AO[3] = {start[0] - c.p1[0], start[1] - c.p1[1], start[2] - c.p1[2]};
    auto cross = [](const double* u, const double* v, double* r) {
        r[0] = u[1] * v[2] - u[2] * v[1];
        r[1] = u[2] * v[0] - u[0] * v[2];
        r[2] = u[0] * v[1] - u[1] * v[0];
    };
    auto dot = [](const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    double AOxAB[3], VxAB[3];
    cross(AO, AB, AOxAB);
    cross(dir, AB, VxAB);
    const double ab2 = dot(AB, AB);
    const double qa = dot(VxAB, VxAB);
    const double qb = 2 * dot(VxAB, AOxAB);
    const double qc = dot(AOxAB, AOxAB) - (c.R * c.R * ab2);
    const double disc = qb * qb - 4 * qa * qc;
    if (disc < 0) return 0.0;
    const double t = (-qb - sqrt(disc)) / (2 * qa);
    if (t < 0) return 0.0;
    return t;
}

// Entries: interior non-wall nodes and their links ending on a curved node, with the
// delta of LB::initializeCurved (LB.cpp:589-603) for the wall node's link back to the
// node (a wall node on the boundary layer links to itself: delta stays 0) and the wall
// node's velocity: the speed of the wall whose plane holds it, else of the cylinder it is
// outside of (solid index), else zero (LB.cpp:969-990; walls built from boundary codes
// do not move).
__global__ void k_curved_list(CurvedArgs a, const double* p2s) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N || !interior(a, i)) return;
    const uint8_t t = a.ntype[i] & HB_TYPE_MASK;
    if (t >= 5 && t <= 9) return;
    for (int j = 1; j < Q; ++j) {
        const long long w = link_of(a, i, j);
        if ((a.ntype[w] & HB_TYPE_MASK) != HB_T_CURVED) continue;
        CurvedEntry e;
        e.i = (uint32_t)i;
        e.back = (uint32_t)link_of(a, i, opp(j));
        e.j = j;
        e.delta = 0.0;
        double pw[3];
        pos_of(a, w, pw);
        if (interior(a, w)) {  // d[w][opp j] is this (non-wall) node
            const double dir[3] = {(double)cx(opp(j)), (double)cy(opp(j)), (double)cz(opp(j))};
            e.delta = 1.0 - segment_intercept(a.cyl[0], pw, dir, p2s);
        }
        e.v[0] = e.v[1] = e.v[2] = 0.0;
        const uint32_t s = a.solid[w];
        bool in_wall = false;
        if ((int)s < a.nw) {
            const double d = a.wn[s][0] * (pw[0] - a.wp[s][0]) + a.wn[s][1] * (pw[1] - a.wp[s][1]) +
                             a.wn[s][2] * (pw[2] - a.wp[s][2]);
            in_wall = d < 0.0;
        }
        if (!in_wall && (int)s < a.ncyl && !inside_cyl(a.cyl[s], pw) && a.cyl[s].moving) {
            // cylinder::getSpeed (utils.cpp:106-120): omega x (distance from the axis)
            const CylDev& c = a.cyl[s];
            const double q[3] = {pw[0] - c.p1[0], pw[1] - c.p1[1], pw[2] - c.p1[2]};
            const double s1 = c.naxes[0] * q[0] + c.naxes[1] * q[1] + c.naxes[2] * q[2];
            const double pp[3] = {c.p1[0] + s1 * c.naxes[0], c.p1[1] + s1 * c.naxes[1], c.p1[2] + s1 * c.naxes[2]};
            const double r[3] = {pw[0] - pp[0], pw[1] - pp[1], pw[2] - pp[2]};
            e.v[0] = c.omega[1] * r[2] - c.omega[2] * r[1];
            e.v[1] = c.omega[2] * r[0] - c.omega[0] * r[2];
            e.v[2] = c.omega[0] * r[1] - c.omega[1] * r[0];
        }
        const int k = atomicAdd(a.count, 1);
        if (k < a.cap) a.list[k] = e;
    }
}

// nodes the rule reads the velocity of: the lattice kernels write their FP64 u
__global__ void k_curved_mark(CurvedArgs a, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    a.ntype[a.list[k].i] |= HB_MIRROR;
    a.ntype[a.list[k].back] |= HB_MIRROR;
}

template <class P>
__global__ void k_curved(CurvedArgs a, int n) {
    using S = typename P::S;
    using T = typename P::T;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const CurvedEntry e = a.list[k];
    const long long i = e.i;
    if (!is_active(a.ntype[i])) return;
    const int j = e.j, o = opp(j);
    S* f = reinterpret_cast<S*>(a.f);
    double fs = (double)P::load(f + (long long)o * a.N + i);  // fs[j], bounced back by the lattice kernel
    if (P::DEV) fs += wgt(o);
    const double nn = a.rho[i];
    const double u[3] = {a.u[i], a.u[a.N + i], a.u[2 * a.N + i]};
    const double visc = a.visc_kind == 1 ? (double)reinterpret_cast<const float*>(a.visc)[i]
                        : a.visc_kind == 2 ? reinterpret_cast<const double*>(a.visc)[i] : a.init_visc;
    const double c[3] = {(double)cx(j), (double)cy(j), (double)cz(j)};
    const double w = wgt(j);
    const double BBi = 2.0 * 3.0 * 1.0 * 1.0 * nn * w * (e.v[0] * c[0] + e.v[1] * c[1] + e.v[2] * c[2]);
    const double tau = 0.5 + 3.0 * visc;
    const double chi = e.delta >= 0.5 ? (2.0 * e.delta - 1.0) / tau : (2.0 * e.delta - 1.0) / (tau - 2.0);
    double ubf[3] = {0.0, 0.0, 0.0};
    if (e.delta >= 0.5) {
        const double m1 = (e.delta - 1) / e.delta, m2 = 1 / e.delta;
        for (int q = 0; q < 3; ++q) ubf[q] = m1 * u[q] + m2 * e.v[q];
    } else if ((a.ntype[e.back] & HB_TYPE_MASK) == HB_T_FLUID) {
        for (int q = 0; q < 3; ++q) ubf[q] = a.u[(long long)q * a.N + e.back];
    } else {
        for (int q = 0; q < 3; ++q) ubf[q] = e.v[q];
    }
    const double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double vu = u[0] * c[0] + u[1] * c[1] + u[2] * c[2];
    const double cu = c[0] * ubf[0] + c[1] * ubf[1] + c[2] * ubf[2];
    const double fstar = nn * w * (1 + 3.0 * cu + 4.5 * vu * vu + 1.5 * usq);  // LB.cpp:1147-1149, 1310
    double fn = (1.0 - chi) * fs + chi * fstar - BBi;
    if (P::DEV) fn -= wgt(o);
    P::store(f + (long long)o * a.N + i, (T)fn);
}

static CurvedArgs curved_args(hb_ctx* c) {
    CurvedArgs a = {};
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype;
    a.solid = c->solid;
    a.ncyl = (int)c->cyl.size();
    for (int k = 0; k < a.ncyl && k < MAX_CYL; ++k) {
        const hb_cyl_host& h = c->cyl[k];
        const double ax[3] = {h.p2[0] - h.p1[0], h.p2[1] - h.p1[1], h.p2[2] - h.p1[2]};
        const double nrm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);  // cylinder::initAxes
        for (int q = 0; q < 3; ++q) {
            a.cyl[k].p1[q] = h.p1[q];
            a.cyl[k].naxes[q] = ax[q] / nrm;
            a.cyl[k].omega[q] = h.omega[q];
        }
        a.cyl[k].R = h.R;
        a.cyl[k].moving = h.moving;
    }
    a.nw = c->d.nw;
    for (int w = 0; w < MAX_WALLS; ++w)
        for (int q = 0; q < 3; ++q) {
            a.wp[w][q] = w < c->d.nw ? c->d.wall_p[w][q] : 0.0;
            a.wn[w][q] = w < c->d.nw ? c->d.wall_n[w][q] : 0.0;
        }
    a.list = reinterpret_cast<CurvedEntry*>(c->curved_list);
    a.count = c->curved_cnt;
    a.cap = c->curved_n;
    a.rho = c->rho;
    a.u = c->u;
    a.visc = c->visc;
    a.visc_kind = c->visc ? (c->P.precision == HB_FP64 ? 2 : 1) : 0;
    a.init_visc = c->P.init_visc;
    return a;
}

void launch_init_cylinders(hb_ctx* c) {
    if (c->cyl.empty()) return;
    const CurvedArgs a = curved_args(c);
    k_cyl_types<<<(unsigned)ceil_div(c->N, 256), 256, 0, c->stream>>>(a);
}

int curved_init(hb_ctx* c) {
    c->curved_n = 0;
    if (c->cyl.empty()) return 0;
    if (!c->curved_cnt && cudaMalloc(&c->curved_cnt, sizeof(int)) != cudaSuccess) return -1;
    double* p2s = nullptr;
    if (cudaMalloc(&p2s, 3 * sizeof(double)) != cudaSuccess) return -1;
    cudaMemcpy(p2s, c->cyl[0].p2, 3 * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(c->curved_cnt, 0, sizeof(int));
    CurvedArgs a = curved_args(c);
    a.list = nullptr;
    a.cap = 0;
    const unsigned G = (unsigned)ceil_div(c->N, 256);
    k_curved_list<<<G, 256, 0, c->stream>>>(a, p2s);
    int n = 0;
    cudaMemcpyAsync(&n, c->curved_cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    if (n > 0) {
        if (c->curved_list) cudaFree(c->curved_list);
        if (cudaMalloc(&c->curved_list, sizeof(CurvedEntry) * n) != cudaSuccess) { cudaFree(p2s); return -1; }
        c->curved_n = n;
        a = curved_args(c);
        cudaMemsetAsync(c->curved_cnt, 0, sizeof(int), c->stream);
        k_curved_list<<<G, 256, 0, c->stream>>>(a, p2s);
        k_curved_mark<<<(unsigned)ceil_div(n, 128), 128, 0, c->stream>>>(a, n);
        cudaStreamSynchronize(c->stream);
    }
    cudaFree(p2s);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// the MIRROR bits after a host upload rewrote the node bytes
void curved_remark(hb_ctx* c) {
    if (c->curved_n == 0) return;
    const CurvedArgs a = curved_args(c);
    k_curved_mark<<<(unsigned)ceil_div(c->curved_n, 128), 128, 0, c->stream>>>(a, c->curved_n);
}

void launch_curved(hb_ctx* c, void* f) {
    if (c->curved_n == 0) return;
    CurvedArgs a = curved_args(c);
    a.f = f;
    const unsigned G = (unsigned)ceil_div(c->curved_n, 128);
    if (c->P.precision == HB_FP64) k_curved<PolF64><<<G, 128, 0, c->stream>>>(a, c->curved_n);
    else if (c->P.precision == HB_FP32) k_curved<PolF32><<<G, 128, 0, c->stream>>>(a, c->curved_n);
    else k_curved<PolF16><<<G, 128, 0, c->stream>>>(a, c->curved_n);
}

}  // namespace hb
