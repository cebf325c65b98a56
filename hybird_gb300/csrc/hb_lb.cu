// hb_lb.cu -- fused D3Q19 collide+stream kernel, lattice init and lattice up/download.
//
// The reference updates each active node as reconstruct -> hydro force -> collide ->
// store -> pull-stream (LB.cpp:221-233, 1062-1488).  Here one kernel does all of it in
// PUSH form: the node reads its own 19 post-streaming populations (coalesced SoA loads),
// collides in registers and scatters the post-collision values to the neighbours that
// pull them in the reference.  Links to non-active neighbours are resolved by the node
// itself, exactly as the reference's pull rules: static wall -> bounce-back
// (LB.cpp:1344-1356), moving wall -> bounce-back with 6 n w (u_w.c) (LB.cpp:1321-1341),
// gas -> constant-pressure reconstruction (LB.cpp:1237-1246).  Every population of
// every active node is written exactly once per step, so the state between steps is the
// reference's node::f after streaming, and the free-surface and coupling phases, which
// the reference runs between streaming and the next collision, see the same data.
//
// This file holds the FP64 form, which follows the reference's arithmetic order and is
// compiled without FMA contraction (as the reference's x86 build computes), plus lattice
// init and up/download; the FP32 / FP16-storage form is in hb_lb32.cu.
//
// Roofline: per lattice update the kernel reads 19 and writes 19 stored populations
// plus the one-byte node type: 2*19*s + 1 bytes (s = 8, 4, 2 for FP64, FP32, FP16S).
#include <algorithm>
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {


// neighbour of interior node (x,y,z) along direction j with the reference's periodic
// remap (LB.cpp:437-472): a link crossing a periodic face re-enters on the opposite side
__device__ __forceinline__ long long link_index(const LBArgs& a, int x, int y, int z, int j) {
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && a.per[0]) xn = a.X - 2;
    else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2;
    else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2;
    else if (zn == a.Z - 1 && a.per[5]) zn = 1;
    return (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
}

// Moving bounce-back: velocity of particle p's solid at node (x, y, z), the element's
// velocity plus its spin times the lever arm from the element centre (the reference's
// commented particle branch, LB.cpp:1247-1276: radius = node - x0 + radiusVec)
__device__ __forceinline__ void mbb_velocity(const Particles& q, int p, int x, int y, int z, double& vx, double& vy,
                                             double& vz) {
    const int E = q.count;
    const double rx = (double)x - q.x0[p], ry = (double)y - q.x0[E + p], rz = (double)z - q.x0[2 * E + p];
    const double wx = q.w[p], wy = q.w[E + p], wz = q.w[2 * E + p];
    vx = q.x1[p] + (wy * rz - wz * ry);
    vy = q.x1[E + p] + (wz * rx - wx * rz);
    vz = q.x1[2 * E + p] + (wx * ry - wy * rx);
}

template <class P>
__global__ void __launch_bounds__(256) k_collide_stream(LBArgs a) {
    using T = typename P::T;
    using S = typename P::S;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1;
    const int z = blockIdx.z + 1;
    if (x < 1 || x > a.X - 2) return;
    const long long N = a.N;
    const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
    const uint8_t t = a.ntype[i];
    if (!is_fluid(t, a.mbb)) return;
    const int mode = *a.mode;
    const S* fin = reinterpret_cast<const S*>(a.fin);
    S* fout = reinterpret_cast<S*>(a.fout);
    const uint8_t code = t & HB_TYPE_MASK;

    T f[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) f[j] = P::load(fin + (long long)j * N + i);

    // ---- reconstruct (node.cpp:63-83); deviation forms keep rho-1 to preserve digits
    T n, dn;
    {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < Q; ++j) s += f[j];
        if constexpr (P::DEV) { dn = s; n = T(1) + s; }
        else { n = s; dn = s - T(1); }
    }
    T mx = T(0), my = T(0), mz = T(0);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        if (cx(j) > 0) mx += f[j]; else if (cx(j) < 0) mx += -f[j];
        if (cy(j) > 0) my += f[j]; else if (cy(j) < 0) my += -f[j];
        if (cz(j) > 0) mz += f[j]; else if (cz(j) < 0) mz += -f[j];
    }
    T ux = mx / n, uy = my / n, uz = mz / n;
    if (!(n > T(0)) || ux != ux || uy != uy || uz != uz) flag_status(a.status, 0);

    // ---- direct-forcing coupling (LB.cpp:1863-1904): node force -eps (u - u_p)
    T hx = T(0), hy = T(0), hz = T(0);
    const double m_i = a.free_surface ? a.mass[i] : 1.0;
    if (a.couple && (t & HB_INSIDE)) {
        int p = (int)a.solid[i];
        const int E = a.parts.count;
        double cxp, cyp, czp;
        if (a.parts.pkey) {  // a particle of an element or a ghost: its element's centre (+ shift)
            const long long st = a.parts.pstride;
            cxp = a.parts.pcen[p]; cyp = a.parts.pcen[st + p]; czp = a.parts.pcen[2 * st + p];
            p = a.parts.pkey[p];
        } else {
            cxp = a.parts.x0[p]; cyp = a.parts.x0[E + p]; czp = a.parts.x0[2 * E + p];
        }
        const double rx = (double)x - cxp;
        const double ry = (double)y - cyp;
        const double rz = (double)z - czp;
        const double wx = a.parts.w[p], wy = a.parts.w[E + p], wz = a.parts.w[2 * E + p];
        const double lvx = a.parts.x1[p] + (wy * rz - wz * ry);
        const double lvy = a.parts.x1[E + p] + (wz * rx - wx * rz);
        const double lvz = a.parts.x1[2 * E + p] + (wx * ry - wy * rx);
        const T lf = T(m_i / (double)n);
        const T dvx = lf * (ux - T(lvx)), dvy = lf * (uy - T(lvy)), dvz = lf * (uz - T(lvz));
        hx = T(0) + T(-1) * dvx;
        hy = T(0) + T(-1) * dvy;
        hz = T(0) + T(-1) * dvz;
        T* dv = reinterpret_cast<T*>(a.dv);
        dv[i] = dvx;
        dv[N + i] = dvy;
        dv[2 * N + i] = dvz;
    }

    // ---- collision (LB.cpp:1094-1111, node.cpp:85-184)
    const T Fx = T(a.F[0]) + hx, Fy = T(a.F[1]) + hy, Fz = T(a.F[2]) + hz;
    ux = ux + (T(0.5) * Fx) / n;  // shiftVelocity
    uy = uy + (T(0.5) * Fy) / n;
    uz = uz + (T(0.5) * Fz) / n;
    const T usq = ux * ux + uy * uy + uz * uz;
    T feq[Q];  // FP64: f_eq; deviation forms: f_eq - w
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        T vu = T(0);
        if (cx(j) > 0) vu += ux; else if (cx(j) < 0) vu += -ux;
        if (cy(j) > 0) vu += uy; else if (cy(j) < 0) vu += -uy;
        if (cz(j) > 0) vu += uz; else if (cz(j) < 0) vu += -uz;
        const T w = T(wgt(j));
        if constexpr (P::DEV)
            feq[j] = w * (dn + n * (T(3) * vu + T(4.5) * vu * vu - T(1.5) * usq));
        else
            feq[j] = w * n * (T(1) + T(3) * vu + T(4.5) * vu * vu - T(1.5) * usq);
    }
    T visc;
    if (a.visc_model) {  // computeShearRate (node.cpp:103-145)
        T* vp = reinterpret_cast<T*>(a.visc);
        const T vold = vp[i];
        const T tau = T(0.5) + T(3) * vold;
        T gxx = 0, gyy = 0, gzz = 0, gxy = 0, gxz = 0, gyz = 0;
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const T d = f[j] - feq[j];
            if (cx(j)) gxx += d;
            if (cy(j)) gyy += d;
            if (cz(j)) gzz += d;
            if (cx(j) * cy(j) > 0) gxy += d; else if (cx(j) * cy(j) < 0) gxy += -d;
            if (cx(j) * cz(j) > 0) gxz += d; else if (cx(j) * cz(j) < 0) gxz += -d;
            if (cy(j) * cz(j) > 0) gyz += d; else if (cy(j) * cz(j) < 0) gyz += -d;
        }
        const T sc = T(1.5) / (tau * n);
        gxx *= sc; gyy *= sc; gzz *= sc; gxy *= sc; gxz *= sc; gyz *= sc;
        const T shear = sqrt(T(0.5) * (gxx * gxx + gyy * gyy + gzz * gzz +
                                       T(2) * (gxy * gxy + gxz * gxz + gyz * gyz)));
        const T nuTurb = (a.visc_model & 2) ? T(a.turb_const) * shear : T(0);
        const T nuApp = (a.visc_model & 1) ? T(a.plastic_visc) + T(a.yield_stress) / (n * T(2) * shear) : vold;
        const T minV = T((0.501 - 0.5) / 3.0), maxV = T((1.8 - 0.5) / 3.0);
        visc = fmax(minV, fmin(maxV, nuApp + nuTurb));  // NaN -> maxV like std::min/max
        vp[i] = visc;
    } else {
        visc = T(a.init_visc);
    }
    T fs[Q];
    if (a.collision == HB_TRT) {
        const T tp = T(0.5) + T(3) * visc;
        const T tm = T(a.trt_magic) / (tp - T(0.5)) + T(0.5);
        const T wp = T(1) / tp, wm = T(1) / tm;
        const T ap = T(1) - T(0.5) * wp, am = T(1) - T(0.5) * wm;
        T Fi[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const T vu = T(cx(j)) * ux + T(cy(j)) * uy + T(cz(j)) * uz;
            const T fpx = T(9) * vu * T(cx(j)) + T(3) * (T(cx(j)) - ux);
            const T fpy = T(9) * vu * T(cy(j)) + T(3) * (T(cy(j)) - uy);
            const T fpz = T(9) * vu * T(cz(j)) + T(3) * (T(cz(j)) - uz);
            Fi[j] = T(wgt(j)) * (fpx * Fx + fpy * Fy + fpz * Fz);
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const int o = opp(j);
            const T fp = T(0.5) * (f[j] + f[o]), fm = T(0.5) * (f[j] - f[o]);
            const T ep = T(0.5) * (feq[j] + feq[o]), em = T(0.5) * (feq[j] - feq[o]);
            fs[j] = f[j] - wp * (fp - ep) - wm * (fm - em) + ap * T(0.5) * (Fi[j] + Fi[o]) +
                    am * T(0.5) * (Fi[j] - Fi[o]);
        }
    } else {
        const T omega = T(1) / (T(0.5) + T(3) * visc);
        const T omegaf = T(1) - T(1) / (T(1) + T(6) * visc);
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            T v = f[j] + omega * (feq[j] - f[j]);  // solveCollision
            T vu = T(0);
            if (cx(j) > 0) vu += ux; else if (cx(j) < 0) vu += -ux;
            if (cy(j) > 0) vu += uy; else if (cy(j) < 0) vu += -uy;
            if (cz(j) > 0) vu += uz; else if (cz(j) < 0) vu += -uz;
            const T fpx = T(9) * vu * T(cx(j)) + T(3) * (T(cx(j)) - ux);  // addForce
            const T fpy = T(9) * vu * T(cy(j)) + T(3) * (T(cy(j)) - uy);
            const T fpz = T(9) * vu * T(cz(j)) + T(3) * (T(cz(j)) - uz);
            v += T(1) * omegaf * T(wgt(j)) * (fpx * Fx + fpy * Fy + fpz * Fz);
            fs[j] = v;
        }
    }

    // ---- node macros needed by later phases (free surface, downloads, wall force)
    const bool all = (mode & 1) != 0;
    if (all || a.free_surface || !(t & HB_BULK)) a.rho[i] = (double)n;
    if (all || code == HB_T_INTERFACE || (t & HB_MIRROR)) {
        a.u[i] = (double)ux; a.u[N + i] = (double)uy; a.u[2 * N + i] = (double)uz;
        a.hf[i] = (double)hx; a.hf[N + i] = (double)hy; a.hf[2 * N + i] = (double)hz;
    }

    // ---- streaming (push form of LB.cpp:1216-1463)
    P::store(fout + i, fs[0]);
    if (t & HB_BULK) {
#pragma unroll
        for (int j = 1; j < Q; ++j) P::store(fout + (long long)j * N + link_index(a, x, y, z, j), fs[j]);
        return;
    }
#pragma unroll
    for (int j = 1; j < Q; ++j) {
        const long long l = link_index(a, x, y, z, j);
        const uint8_t tl = a.ntype[l];
        const uint8_t lc = tl & HB_TYPE_MASK;
        const int o = opp(j);
        if (a.mbb && (tl & HB_INSIDE) && (lc == HB_T_FLUID || lc == HB_T_INTERFACE)) {
            // moving bounce-back on a particle (no wrapped links: particles with
            // periodic faces are not taken in this mode), as the moving wall's rule
            double ubx, uby, ubz;
            mbb_velocity(a.parts, (int)a.solid[l], x + cx(j), y + cy(j), z + cz(j), ubx, uby, ubz);
            const double uw = ubx * cx(j) + uby * cy(j) + ubz * cz(j);
            const T BBi = T(6.0 * (double)n * wgt(j) * uw);
            P::store(fout + (long long)o * N + i, fs[j] - BBi);
        } else if (lc == HB_T_FLUID || lc == HB_T_INTERFACE) {
            P::store(fout + (long long)j * N + l, fs[j]);
        } else if (lc == HB_T_GAS) {
            T vu = T(0);
            if (cx(j) > 0) vu += ux; else if (cx(j) < 0) vu += -ux;
            if (cy(j) > 0) vu += uy; else if (cy(j) < 0) vu += -uy;
            if (cz(j) > 0) vu += uz; else if (cz(j) < 0) vu += -uz;
            const T w = T(wgt(j));
            T v;
            if constexpr (P::DEV) v = -fs[j] + w * (T(9) * (vu * vu) - T(3) * usq);
            else v = -fs[j] + w * T(1) * (T(2) + T(9) * (vu * vu) - T(3) * usq);
            P::store(fout + (long long)o * N + i, v);
        } else if (lc == HB_T_DYNWALL) {
            const double uw = a.u[l] * cx(j) + a.u[N + l] * cy(j) + a.u[2 * N + l] * cz(j);
            const T BBi = T(6.0 * (double)n * wgt(j) * uw);
            P::store(fout + (long long)o * N + i, fs[j] - BBi);
        } else if (lc == HB_T_STATWALL || lc == HB_T_SLIPSTAT || lc == HB_T_SLIPDYN || lc == HB_T_CURVED) {
            P::store(fout + (long long)o * N + i, fs[j]);  // slip / curved walls: completed afterwards
        } else {
            flag_status(a.status, 1);  // TYPE ERROR (LB.cpp:1458-1461)
        }
    }
}

// Moving-wall momentum exchange and extra mass (LB.cpp:1321-1341): recomputed from the
// post-streaming populations, f_out[opp j] = fs[j] - BBi, so the hot kernel stays free
// of reductions.  One FP64 partial per CTA and wall, summed in CTA order afterwards.
template <class P>
__global__ void __launch_bounds__(256) k_wallforce(LBArgs a) {
    using S = typename P::S;
    __shared__ double sh[256];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1, z = blockIdx.z + 1;
    const long long N = a.N;
    double acc[MAX_WALLS * 3 + 1];
#pragma unroll
    for (int k = 0; k < MAX_WALLS * 3 + 1; ++k) acc[k] = 0.0;
    if (x >= 1 && x <= a.X - 2) {
        const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
        const uint8_t t = a.ntype[i];
        if (is_fluid(t, a.mbb) && !(t & HB_BULK)) {
            const S* fcur = reinterpret_cast<const S*>(a.fout);
            for (int j = 1; j < Q; ++j) {
                const long long l = link_index(a, x, y, z, j);
                if ((a.ntype[l] & HB_TYPE_MASK) != HB_T_DYNWALL) continue;
                const double uw = a.u[l] * cx(j) + a.u[N + l] * cy(j) + a.u[2 * N + l] * cz(j);
                const double BBi = 6.0 * a.rho[i] * wgt(j) * uw;
                double fo = (double)P::load(fcur + (long long)opp(j) * N + i);
                if (P::DEV) fo += wgt(j);
                const double fsj = fo + BBi;
                const double sc = (2.0 * (fsj - 1.0 * wgt(j)) - BBi) * 1.0;
                const int w = (int)a.solid[l];
                if (w >= 0 && w < MAX_WALLS) {
                    acc[3 * w] += sc * cx(j);
                    acc[3 * w + 1] += sc * cy(j);
                    acc[3 * w + 2] += sc * cz(j);
                }
                acc[MAX_WALLS * 3] += BBi * a.mass[i];
            }
        }
    }
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    for (int k = 0; k < MAX_WALLS * 3 + 1; ++k) {
        sh[threadIdx.x] = acc[k];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) a.wall_part[(long long)k * nb + b] = sh[0];
        __syncthreads();
    }
}

__global__ void k_wallforce_final(const double* part, int nb, double* out) {
    const int k = threadIdx.x;
    if (k >= MAX_WALLS * 3 + 1) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(long long)k * nb + b];
    out[k] = s;
}


// ---- initialisation ------------------------------------------------------------------

struct InitArgs {
    int X, Y, Z;
    long long N;
    int boundary[6];
    int nw;
    double wp[MAX_WALLS][3], wn[MAX_WALLS][3];
    int wcode[MAX_WALLS];
    double gas_x, gas_z;
    int mbb;  // moving bounce-back: nodes inside particles are solid
};

// lattice boundary codes (LB.cpp:393-432), DEM walls (LB.cpp:497-533)
__global__ void k_init_types(InitArgs a, uint8_t* ntype, uint32_t* solid) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    auto wall = [](int c) { return c >= 5 && c <= 9; };
    int t = HB_T_FLUID;
    if (x == 0 && !wall(t)) t = a.boundary[0];
    else if (x == a.X - 1 && !wall(t)) t = a.boundary[1];
    if (y == 0 && !wall(t)) t = a.boundary[2];
    else if (y == a.Y - 1 && !wall(t)) t = a.boundary[3];
    if (z == 0 && !wall(t)) t = a.boundary[4];
    else if (z == a.Z - 1 && !wall(t)) t = a.boundary[5];
    uint32_t s = 0;
    for (int w = 0; w < a.nw; ++w) {
        const double d = a.wn[w][0] * ((double)x - a.wp[w][0]) + a.wn[w][1] * ((double)y - a.wp[w][1]) +
                         a.wn[w][2] * ((double)z - a.wp[w][2]);
        if (d < 0.0) {
            s = (uint32_t)w;
            t = a.wcode[w];
        }
    }
    ntype[i] = (uint8_t)t;
    solid[i] = s;
}

// particle flags, last particle in list order wins (LB.cpp:475-495).  On the
// per-particle path (periodic faces, multi-sphere elements) the list holds the P
// particles and then the ghosts: centres from px (stride st), radius of the particle's
// element, count P + gmeta[0].
__global__ void k_init_particles(InitArgs a, const double* x0, long long st, const double* r, int P,
                                 const int* pkey, const int* gmeta, const uint8_t* ntype, int* owner) {
    const int p = blockIdx.x;
    if (gmeta && p >= P + gmeta[0]) return;
    const double cxp = x0[p], cyp = x0[st + p], czp = x0[2 * st + p], rr = r[pkey ? pkey[p] : p];
    const int x0i = max(0, (int)floor(cxp - rr) - 1), x1i = min(a.X - 1, (int)ceil(cxp + rr) + 1);
    const int y0i = max(0, (int)floor(cyp - rr) - 1), y1i = min(a.Y - 1, (int)ceil(cyp + rr) + 1);
    const int z0i = max(0, (int)floor(czp - rr) - 1), z1i = min(a.Z - 1, (int)ceil(czp + rr) + 1);
    const int nx = x1i - x0i + 1, ny = y1i - y0i + 1, nz = z1i - z0i + 1;
    for (int k = threadIdx.x; k < nx * ny * nz; k += blockDim.x) {
        const int x = x0i + k % nx, y = y0i + (k / nx) % ny, z = z0i + k / (nx * ny);
        const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
        if (!is_active(ntype[i])) continue;
        const double dx = x - cxp, dy = y - cyp, dz = z - czp;
        if (dx * dx + dy * dy + dz * dz < rr * rr) atomicMax(owner + i, p);
    }
}

// objects become static wall nodes, last object wins (LB.cpp:535-550); particle owner
// commits the inside flag (set before objects in the reference, so it survives them)
__global__ void k_init_objects(InitArgs a, const double* ox, const double* orad, int O,
                               const int* owner, uint8_t* ntype, uint32_t* solid) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    uint8_t t = ntype[i];
    uint32_t s = solid[i];
    if (owner && owner[i] >= 0) {
        t |= HB_INSIDE;
        s = (uint32_t)owner[i];
    }
    for (int o = 0; o < O; ++o) {
        const double dx = x - ox[o], dy = y - ox[O + o], dz = z - ox[2 * O + o];
        if (dx * dx + dy * dy + dz * dz < orad[o] * orad[o]) {
            s = (uint32_t)o;
            t = (t & HB_INSIDE) | HB_T_STATWALL;
        }
    }
    // dam-break column: gas outside x < gx*X, z < gz*Z
    if ((t & HB_TYPE_MASK) == HB_T_FLUID && (a.gas_x > 0.0 || a.gas_z > 0.0)) {
        if ((double)x >= a.gas_x * a.X || (double)z >= a.gas_z * a.Z) t = (t & HB_INSIDE) | HB_T_GAS;
    }
    ntype[i] = t;
    solid[i] = s;
}

__device__ __forceinline__ long long init_link(const InitArgs& a, const int* per, long long i, int j) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && per[0]) xn = a.X - 2; else if (xn == a.X - 1 && per[1]) xn = 1;
    if (yn == 0 && per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && per[3]) yn = 1;
    if (zn == 0 && per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && per[5]) zn = 1;
    return (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
}

struct PerFaces { int v[6]; };

// interface = fluid with a gas link (LB.cpp:788-797)
__global__ void k_init_interface(InitArgs a, PerFaces pf, uint8_t* ntype) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    if (x < 1 || y < 1 || z < 1 || x > a.X - 2 || y > a.Y - 2 || z > a.Z - 2) return;
    const uint8_t t = ntype[i];
    if ((t & HB_TYPE_MASK) != HB_T_FLUID) return;
    for (int j = 1; j < Q; ++j)
        if ((ntype[init_link(a, pf.v, i, j)] & HB_TYPE_MASK) == HB_T_GAS) {
            ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_INTERFACE;
            return;
        }
}

// isolated interface (no fluid link) -> gas (LB.cpp:800-814)
__global__ void k_init_isolated(InitArgs a, PerFaces pf, uint8_t* ntype) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const uint8_t t = ntype[i];
    if ((t & HB_TYPE_MASK) != HB_T_INTERFACE) return;
    for (int j = 1; j < Q; ++j)
        if ((ntype[init_link(a, pf.v, i, j)] & HB_TYPE_MASK) == HB_T_FLUID) return;
    ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_GAS;
}

__global__ void k_active_max(InitArgs a, const uint8_t* ntype, int* mx) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    if (!is_active(ntype[i])) return;
    atomicMax(mx + 0, (int)(i % a.X));
    atomicMax(mx + 1, (int)((i / a.X) % a.Y));
    atomicMax(mx + 2, (int)(i / ((long long)a.X * a.Y)));
}

// hydrostatic variables + f = f_eq (LB.cpp:909-944, node.cpp:26-61) and wall nodes
template <class P>
__global__ void k_init_vars(InitArgs a, LBArgs b, const int* mx, double Fx, double Fy, double Fz,
                            double ivx, double ivy, double ivz, double visc0) {
    using T = typename P::T;
    using S = typename P::S;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const long long N = a.N;
    const uint8_t t = b.ntype[i];
    const uint8_t code = t & HB_TYPE_MASK;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    double n = 1.0, mass = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
    bool node = false;
    if (code == HB_T_FLUID) {
        const double dhx = (double)x - mx[0], dhy = (double)y - mx[1], dhz = (double)z - mx[2];
        n = 1.0 + 3.0 * 1.0 * 1.0 * 1.0 * (dhx * Fx + dhy * Fy + dhz * Fz);
        mass = 1.0;
        vx = ivx; vy = ivy; vz = ivz;
        node = true;
    } else if (code == HB_T_INTERFACE) {
        n = 1.0;
        mass = 0.5 * 1.0;
        vx = ivx; vy = ivy; vz = ivz;
        node = true;
    }
    double ux = 0.0, uy = 0.0, uz = 0.0;
    if (node) {
        ux = 1.0 * Fx / 2.0 / n + vx;
        uy = 1.0 * Fy / 2.0 / n + vy;
        uz = 1.0 * Fz / 2.0 / n + vz;
    }
    b.rho[i] = n;
    b.u[i] = ux; b.u[N + i] = uy; b.u[2 * N + i] = uz;
    b.hf[i] = 0.0; b.hf[N + i] = 0.0; b.hf[2 * N + i] = 0.0;
    b.mass[i] = mass;
    if (b.visc_model) reinterpret_cast<T*>(b.visc)[i] = node ? T(visc0) : T(0);
    S* f = reinterpret_cast<S*>(b.fout);
    const double usq = ux * ux + uy * uy + uz * uz;
    for (int j = 0; j < Q; ++j) {
        const double vu = ux * cx(j) + uy * cy(j) + uz * cz(j);
        double fe = node ? wgt(j) * n * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq) : wgt(j);
        if (P::DEV) fe -= wgt(j);
        P::store(f + (long long)j * N + i, (T)fe);
        P::store(reinterpret_cast<S*>(const_cast<void*>(b.fin)) + (long long)j * N + i, (T)(P::DEV ? 0.0 : wgt(j)));
    }
}

// HB_BULK: node active and all 18 links lead to active nodes
// HB_BULK / HB_PWRAP flags and, for active nodes, the mask of links that are not plain
// (bit j: the neighbour along j is not active, or the link crosses a periodic face); the
// reduced-precision lattice kernel sends only those links through the general push.
// 3D grid (x from the thread, y and z from the block).  With `changed` set, the pass
// runs only when that counter is non-zero (the free surface changed some cell between
// gas and interface) and resets it.
constexpr int BULK_ZC = 8;  // z planes per block of the refresh pass

__device__ __forceinline__ void bulk_node(const InitArgs& a, const PerFaces& pf, uint8_t* ntype,
                                          unsigned long long* lmask, int x, int y, int z) {
    const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
    uint8_t t = ntype[i];
    bool bulk = is_fluid(t, a.mbb);
    bool wrap = false;  // some link crosses a periodic face (checked over all 18 links)
    uint32_t mask = 0;  // links that need the general push
    uint32_t bb = 0;    // links that end on a static wall: plain bounce-back into the node itself
    if (bulk) {
        if (x < 1 || y < 1 || z < 1 || x > a.X - 2 || y > a.Y - 2 || z > a.Z - 2) {
            bulk = false;
            mask = 0x7FFFEu;
        } else {
            // unrolled: the 18 neighbour bytes are loaded together, not one after another
#pragma unroll
            for (int j = 1; j < Q; ++j) {
                int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
                if (xn == 0 && pf.v[0]) xn = a.X - 2; else if (xn == a.X - 1 && pf.v[1]) xn = 1;
                if (yn == 0 && pf.v[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && pf.v[3]) yn = 1;
                if (zn == 0 && pf.v[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && pf.v[5]) zn = 1;
                const bool wj = xn != x + cx(j) || yn != y + cy(j) || zn != z + cz(j);
                const long long l = (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
                const uint8_t tl = ntype[l];
                const bool act = is_fluid(tl, a.mbb);  // a solid particle node takes the general push
                const uint8_t tc = tl & HB_TYPE_MASK;
                if (tc == HB_T_STATWALL || tc == HB_T_SLIPSTAT || tc == HB_T_SLIPDYN || tc == HB_T_CURVED) bb |= 1u << j;
                else if (!act || wj) mask |= 1u << j;
                if (!act) bulk = false;
                if (wj) wrap = true;
            }
        }
    }
    uint8_t nt = bulk ? (t | HB_BULK) : (t & ~HB_BULK);
    nt = wrap ? (nt | HB_PWRAP) : (nt & ~HB_PWRAP);
    if (nt != t) ntype[i] = nt;
    if (lmask) lmask[i] = (unsigned long long)mask | ((unsigned long long)bb << 32);
}

__global__ void k_bulk(InitArgs a, PerFaces pf, uint8_t* ntype, unsigned long long* lmask, int* changed) {
    pdl_enter();
    if (changed && *changed == 0) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.X) return;
    for (int zz = 0; zz < BULK_ZC; ++zz) {
        const int z = blockIdx.z * BULK_ZC + zz;
        if (z < a.Z) bulk_node(a, pf, ntype, lmask, x, y, z);
    }
}

// resets the activity-change counter after the (conditional) refresh has run
__global__ void k_bulk_done(int* changed) {
    pdl_enter();
    *changed = 0;
}

// ---- upload / download ---------------------------------------------------------------

template <class P>
__global__ void k_upload_f(const double* f, long long N, void* dst) {
    using S = typename P::S;
    using T = typename P::T;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int j = 0; j < Q; ++j) {
        double v = f[(long long)j * N + i];
        if (P::DEV) v -= wgt(j);
        P::store(reinterpret_cast<S*>(dst) + (long long)j * N + i, (T)v);
    }
}

template <class P>
__global__ void k_download_f(const void* src, long long N, double* f) {
    using S = typename P::S;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int j = 0; j < Q; ++j) {
        double v = (double)P::load(reinterpret_cast<const S*>(src) + (long long)j * N + i);
        if (P::DEV) v += wgt(j);
        f[(long long)j * N + i] = v;
    }
}

__global__ void k_pack_types(const uint8_t* type, const uint8_t* inside, uint8_t* ntype, long long N) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= N) return;
    ntype[i] = (uint8_t)((type[i] & HB_TYPE_MASK) | (inside[i] ? HB_INSIDE : 0));
}

// ---- host launchers ------------------------------------------------------------------

static InitArgs init_args(hb_ctx* c) {
    InitArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.boundary[k] = c->P.boundary[k];
    a.nw = c->d.nw;
    for (int w = 0; w < MAX_WALLS; ++w) {
        for (int k = 0; k < 3; ++k) {
            a.wp[w][k] = w < c->d.nw ? c->d.wall_p[w][k] : 0.0;
            a.wn[w][k] = w < c->d.nw ? c->d.wall_n[w][k] : 0.0;
        }
        a.wcode[w] = w < c->d.nw ? c->d.wall_code[w] : HB_T_STATWALL;
    }
    a.gas_x = c->P.gas_box[0];
    a.gas_z = c->P.gas_box[1];
    a.mbb = c->P.coupling == HB_MOVING_BB && c->d.E > 0;
    return a;
}

static PerFaces per_faces(hb_ctx* c) {
    PerFaces p;
    for (int k = 0; k < 6; ++k) p.v[k] = c->P.boundary[k] == HB_T_PERIODIC;
    return p;
}

LBArgs lb_args(hb_ctx* c, int cur) {
    LBArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype;
    a.solid = c->solid;
    a.fin = cur ? c->fB : c->fA;
    a.fout = cur ? c->fA : c->fB;
    a.mode = c->mode;
    a.rho = c->rho;
    a.u = c->u;
    a.hf = c->hf;
    a.mass = c->mass;
    a.visc = c->visc;
    a.dv = c->dv;
    a.hacc = c->hacc;
    a.lmask = c->lmask;
    a.F = c->lb_force;
    a.Ff = c->lb_force_f;
    for (int j = 0; j < Q; ++j) {
        a.ne[j] = cx(j) + c->X * (cy(j) + c->Y * cz(j));
        a.jn[j] = (int)(j * c->N);
        a.so[j] = (int)(j * c->N) + a.ne[j];
    }
    a.init_visc_f = (float)c->P.init_visc;
    a.trt_magic_f = (float)c->P.trt_magic;
    a.plastic_visc_f = (float)c->P.plastic_visc;
    a.yield_stress_f = (float)c->P.yield_stress;
    a.turb_const_f = (float)c->P.turb_const;
    a.init_visc = c->P.init_visc;
    a.collision = c->P.collision;
    a.trt_magic = c->P.trt_magic;
    a.visc_model = (c->P.non_newtonian ? 1 : 0) | (c->P.turbulence ? 2 : 0);
    a.plastic_visc = c->P.plastic_visc;
    a.yield_stress = c->P.yield_stress;
    a.turb_const = c->P.turb_const;
    a.free_surface = c->P.free_surface;
    a.mbb = (c->P.dem_solve && c->d.E > 0 && c->P.coupling == HB_MOVING_BB) ? 1 : 0;
    a.couple = (c->P.dem_solve && c->d.E > 0 && !a.mbb) ? 1 : 0;
    a.parts.count = c->d.E;
    a.parts.x0 = c->d.E ? c->d.x[0] : nullptr;
    a.parts.x1 = c->d.E ? c->d.x[1] : nullptr;
    a.parts.w = c->d.E ? c->d.wG : nullptr;
    a.parts.radius = c->d.E ? c->d.rad : nullptr;
    a.parts.pf = c->d.E ? c->d.pf : nullptr;
    a.parts.pkey = c->d.gen ? c->d.pkey : nullptr;
    a.parts.pcen = c->d.gen ? c->d.pcen : nullptr;
    a.parts.pstride = (long long)c->d.P + c->d.gcap;
    a.status = c->status;
    a.wall_part = c->wall_part;
    a.nwalls = c->d.nw;
    return a;
}

static dim3 lb_grid(hb_ctx* c, int& block) {
    block = c->X <= 64 ? 64 : (c->X <= 128 ? 128 : 256);
    return dim3((unsigned)ceil_div(c->X, block), (unsigned)(c->Y - 2), (unsigned)(c->Z - 2));
}

int launch_init_lattice(hb_ctx* c, const double* el_x0, const double* el_r, int E,
                        const double* ob_x0, const double* ob_r, int O) {
    InitArgs a = init_args(c);
    const int B = 256;
    const int G = ceil_div(c->N, B);
    k_init_types<<<G, B, 0, c->stream>>>(a, c->ntype, c->solid);
    int* owner = nullptr;
    if (E > 0) {
        cudaMalloc(&owner, sizeof(int) * c->N);
        cudaMemsetAsync(owner, 0xFF, sizeof(int) * c->N, c->stream);
        if (c->d.gen)
            k_init_particles<<<c->d.P + c->d.gcap, 256, 0, c->stream>>>(a, c->d.px, (long long)c->d.P + c->d.gcap,
                                                                         el_r, c->d.P, c->d.pkey, c->d.gmeta,
                                                                         c->ntype, owner);
        else
            k_init_particles<<<E, 256, 0, c->stream>>>(a, el_x0, E, el_r, E, nullptr, nullptr, c->ntype, owner);
    }
    launch_init_cylinders(c);  // after particles and walls, before objects (LB.cpp:324-337)
    k_init_objects<<<G, B, 0, c->stream>>>(a, ob_x0, ob_r, O, owner, c->ntype, c->solid);
    PerFaces pf = per_faces(c);
    k_init_interface<<<G, B, 0, c->stream>>>(a, pf, c->ntype);
    k_init_isolated<<<G, B, 0, c->stream>>>(a, pf, c->ntype);
    int* mx = nullptr;
    cudaMalloc(&mx, 3 * sizeof(int));
    cudaMemsetAsync(mx, 0, 3 * sizeof(int), c->stream);
    k_active_max<<<G, B, 0, c->stream>>>(a, c->ntype, mx);
    LBArgs b = lb_args(c, 1);  // fout = fA: the initial state lives in buffer 0
    const double* F = c->P.lbF;  // initialisation always uses lbF (LB.cpp:935)
    const double* iv = c->P.init_velocity;
    if (c->P.precision == HB_FP64)
        k_init_vars<PolF64><<<G, B, 0, c->stream>>>(a, b, mx, F[0], F[1], F[2], iv[0], iv[1], iv[2], c->P.init_visc);
    else if (c->P.precision == HB_FP32)
        k_init_vars<PolF32><<<G, B, 0, c->stream>>>(a, b, mx, F[0], F[1], F[2], iv[0], iv[1], iv[2], c->P.init_visc);
    else
        k_init_vars<PolF16><<<G, B, 0, c->stream>>>(a, b, mx, F[0], F[1], F[2], iv[0], iv[1], iv[2], c->P.init_visc);
    k_bulk<<<dim3((unsigned)ceil_div(c->X, 128), (unsigned)c->Y, (unsigned)ceil_div(c->Z, BULK_ZC)), 128, 0,
             c->stream>>>(a, pf, c->ntype, c->lmask, nullptr);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (owner) cudaFree(owner);
    cudaFree(mx);
    return e == cudaSuccess ? 0 : -1;
}

void launch_refresh_bulk(hb_ctx* c, int* changed) {
    InitArgs a = init_args(c);
    launch_pdl(k_bulk, dim3((unsigned)ceil_div(c->X, 128), (unsigned)c->Y, (unsigned)ceil_div(c->Z, BULK_ZC)), 128,
               c->stream, a, per_faces(c), c->ntype, c->lmask, changed);
    if (changed) launch_pdl(k_bulk_done, 1, 1, c->stream, changed);
}

void launch_lb_step(hb_ctx* c, int cur) {
    LBArgs a = lb_args(c, cur);
    int block;
    dim3 g = lb_grid(c, block);
    if (c->P.precision == HB_FP64) {
        k_collide_stream<PolF64><<<g, block, 0, c->stream>>>(a);
    } else {
        if (a.couple || a.mbb) cudaMemsetAsync(c->hacc, 0, sizeof(unsigned long long) * 7 * c->d.E, c->stream);
        launch_lb_step_dev(c, a);
    }
    launch_slip(c, a.fout);    // slip-wall mixing of the bounced-back diagonals (hb_slip.cu)
    launch_curved(c, a.fout);  // curved-wall interpolation of the bounced-back links (hb_curved.cu)
    if (a.mbb && c->P.precision == HB_FP64) launch_mbb_force(c, cur);  // FP32/FP16: in the lattice kernel
}

void launch_lb_wallforce(hb_ctx* c, int cur) {
    LBArgs a = lb_args(c, cur);
    int block;
    dim3 g = lb_grid(c, block);
    if (c->P.precision == HB_FP64) k_wallforce<PolF64><<<g, block, 0, c->stream>>>(a);
    else if (c->P.precision == HB_FP32) k_wallforce<PolF32><<<g, block, 0, c->stream>>>(a);
    else k_wallforce<PolF16><<<g, block, 0, c->stream>>>(a);
    k_wallforce_final<<<1, 32, 0, c->stream>>>(c->wall_part, (int)(g.x * g.y * g.z), c->wall_force);
}


int launch_upload_lattice(hb_ctx* c, const uint8_t* type, const uint8_t* inside,
                          const uint32_t* solid, const double* f, const double* n, const double* u,
                          const double* mass, const double* visc) {
    const long long N = c->N;
    const int B = 256, G = ceil_div(N, B);
    uint8_t *dt = nullptr, *di = nullptr;
    cudaMalloc(&dt, N);
    cudaMalloc(&di, N);
    cudaMemcpyAsync(dt, type, N, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(di, inside, N, cudaMemcpyHostToDevice, c->stream);
    k_pack_types<<<G, B, 0, c->stream>>>(dt, di, c->ntype, N);
    cudaMemcpyAsync(c->solid, solid, sizeof(uint32_t) * N, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->rho, n, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->u, u, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->mass, mass, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    double* df = nullptr;
    cudaMalloc(&df, sizeof(double) * 19 * N);
    if (f) {
        cudaMemcpyAsync(df, f, sizeof(double) * 19 * N, cudaMemcpyHostToDevice, c->stream);
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(dt);
    cudaFree(di);
    // f given: encode; otherwise f_eq(n,u) as node::initialize does (node.cpp:26-61)
    if (!f) {
        std::vector<double> hf((size_t)19 * N);
        for (long long i = 0; i < N; ++i) {
            const double ux = u[i], uy = u[N + i], uz = u[2 * N + i];
            const double usq = ux * ux + uy * uy + uz * uz;
            for (int j = 0; j < Q; ++j) {
                const double vu = ux * cx(j) + uy * cy(j) + uz * cz(j);
                hf[(size_t)j * N + i] = wgt(j) * n[i] * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
            }
        }
        cudaMemcpy(df, hf.data(), sizeof(double) * 19 * N, cudaMemcpyHostToDevice);
    }
    void* dst = c->cur ? c->fB : c->fA;
    if (c->P.precision == HB_FP64) k_upload_f<PolF64><<<G, B, 0, c->stream>>>(df, N, dst);
    else if (c->P.precision == HB_FP32) k_upload_f<PolF32><<<G, B, 0, c->stream>>>(df, N, dst);
    else k_upload_f<PolF16><<<G, B, 0, c->stream>>>(df, N, dst);
    if (c->visc && visc) {
        if (c->P.precision == HB_FP64) {
            cudaMemcpyAsync(c->visc, visc, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
        } else {
            std::vector<float> vf(N);
            for (long long i = 0; i < N; ++i) vf[i] = (float)visc[i];
            cudaMemcpyAsync(c->visc, vf.data(), sizeof(float) * N, cudaMemcpyHostToDevice, c->stream);
            cudaStreamSynchronize(c->stream);
        }
    }
    launch_refresh_bulk(c);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(df);
    return e == cudaSuccess ? 0 : -1;
}

int launch_download_lattice(hb_ctx* c, double* f_dev, int which) {
    const long long N = c->N;
    const void* src = which ? c->fB : c->fA;
    const int B = 256, G = ceil_div(N, B);
    if (c->P.precision == HB_FP64) k_download_f<PolF64><<<G, B, 0, c->stream>>>(src, N, f_dev);
    else if (c->P.precision == HB_FP32) k_download_f<PolF32><<<G, B, 0, c->stream>>>(src, N, f_dev);
    else k_download_f<PolF16><<<G, B, 0, c->stream>>>(src, N, f_dev);
    return 0;
}

// ---- moving bounce-back coupling (hb_params.coupling = HB_MOVING_BB) ------------------
// Not in the reference (its particle branch is commented out, LB.cpp:1247-1276).  The
// coupling masks (LB.cpp:1921-2033 rules) decide which nodes are inside a particle; here
// those nodes are solid.  After the masks: every node a particle uncovered is refilled
// with the equilibrium of the particle's local velocity at the mean density of its fluid
// links, and the bulk bit / link masks of the changed nodes and their neighbours are
// recomputed.  After the lattice step: each particle's force and torque from the
// bounce-back links into it.  Particles with periodic faces are not taken in this mode,
// so no link wraps.

struct MbbArgs {
    int X, Y, Z;
    long long N;
    uint8_t* ntype;
    uint32_t* solid;
    void* f;                 // population buffer (refill: the current state; force: after streaming)
    double* rho;
    Particles parts;
    const uint32_t* pop;     // nodes uncovered in this step
    const int* npop;
    double* pop_rho;
    const uint32_t* claims;  // (node, particle) pairs covered in this step
    const int* nclaim;
    double *FH, *MH, *fvol;  // element sums (single spheres: element = particle)
};

// One thread per uncovered node: rho = mean density of its fluid links that were fluid
// before this step (popped nodes carry NaN density until their refill is committed), in
// link order, 1 without any; f = f_eq(rho, u) with u the particle's velocity at the node.
template <class P>
__device__ __forceinline__ void mbb_refill_one(const MbbArgs& a, int k) {
    using S = typename P::S;
    using T = typename P::T;
    const long long l = a.pop[k];
    if (a.ntype[l] & HB_INSIDE) return;  // covered again in the same step
    const int x = (int)(l % a.X), y = (int)((l / a.X) % a.Y), z = (int)(l / ((long long)a.X * a.Y));
    double sum = 0.0;
    int cnt = 0;
    // unrolled: the 18 neighbours' bytes and densities are loaded together; the sum still
    // runs in link order
#pragma unroll
    for (int j = 1; j < Q; ++j) {
        const long long m = (long long)(x + cx(j)) + (long long)a.X * ((long long)(y + cy(j)) + (long long)a.Y * (z + cz(j)));
        const double r = a.rho[m];
        if (!is_fluid(a.ntype[m], 1) || r != r) continue;
        sum += r;
        ++cnt;
    }
    const double rho = cnt ? sum / (double)cnt : 1.0;
    double ux, uy, uz;
    mbb_velocity(a.parts, (int)a.solid[l], x, y, z, ux, uy, uz);
    // f_eq in the storage policy's arithmetic (double for FP64 populations, float for the
    // FP32 and FP16 forms, whose stored values carry float precision at most)
    const T rt = (T)rho, uxt = (T)ux, uyt = (T)uy, uzt = (T)uz;
    const T usq = uxt * uxt + uyt * uyt + uzt * uzt;
    S* f = reinterpret_cast<S*>(a.f);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        const T vu = uxt * T(cx(j)) + uyt * T(cy(j)) + uzt * T(cz(j));
        T v = T(wgt(j)) * rt * (T(1) + T(3) * vu + T(4.5) * vu * vu - T(1.5) * usq);
        if (P::DEV) v -= T(wgt(j));
        P::store(f + (long long)j * a.N + l, v);
    }
    a.pop_rho[k] = rho;
}

template <class P>
__global__ void k_mbb_refill_gs(MbbArgs a) {
    pdl_enter();
    const int n = *a.npop;
    // consecutive entries to different blocks: a list of a few hundred nodes reaches
    // every SM (its FP64 work would otherwise queue on the first two)
    for (int k = blockIdx.x + gridDim.x * threadIdx.x; k < n; k += gridDim.x * blockDim.x) mbb_refill_one<P>(a, k);
}

// One thread per (changed node, node or one of its 18 links): the bulk bit and link mask of
// that node from its neighbours' final state; uncovered nodes take their refill density.
// Nodes reached from several changed nodes compute the same values.
__global__ void k_mbb_relink_gs(MbbArgs m, InitArgs a, PerFaces pf, unsigned long long* lmask) {
    pdl_enter();
    const long long np = *m.npop, nc = *m.nclaim;
    const long long total = (np + nc) * Q;
    for (long long t = blockIdx.x + (long long)gridDim.x * threadIdx.x; t < total;  // spread over the blocks
         t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / Q;
        const int j = (int)(t - e * Q);
        const long long l = e < np ? (long long)m.pop[e] : (long long)m.claims[2 * (e - np)];
        const int x = (int)(l % a.X), y = (int)((l / a.X) % a.Y), z = (int)(l / ((long long)a.X * a.Y));
        const int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
        if (xn < 0 || yn < 0 || zn < 0 || xn >= a.X || yn >= a.Y || zn >= a.Z) continue;
        bulk_node(a, pf, m.ntype, lmask, xn, yn, zn);
        if (j == 0 && e < np && !(m.ntype[l] & HB_INSIDE)) m.rho[l] = m.pop_rho[e];
    }
}

// Element force and torque of the FP64 form (node::bounceBackForce, node.cpp:283-291; the
// FP32/FP16 forms sum them inside the lattice kernel): one block per particle over its box; each fluid node's links into the particle contribute
// (2 (fs_j - w_j) - BBi) c_j with fs_j = f_out[opp j] + BBi recovered from the streamed
// state and its moment about the element centre; the solid nodes count the volume.
// Fixed node-to-thread assignment and a fixed tree: the sums are reproducible.
template <class P>
__global__ void __launch_bounds__(256) k_mbb_force(MbbArgs a) {
    using S = typename P::S;
    __shared__ double sh[7][256];
    const int p = blockIdx.x, E = a.parts.count;
    const double cxp = a.parts.x0[p], cyp = a.parts.x0[E + p], czp = a.parts.x0[2 * E + p], r = a.parts.radius[p];
    const int x0 = max(1, (int)floor(cxp - r) - 2), x1 = min(a.X - 2, (int)ceil(cxp + r) + 2);
    const int y0 = max(1, (int)floor(cyp - r) - 2), y1 = min(a.Y - 2, (int)ceil(cyp + r) + 2);
    const int z0 = max(1, (int)floor(czp - r) - 2), z1 = min(a.Z - 2, (int)ceil(czp + r) + 2);
    const int nx = x1 - x0 + 1, ny = y1 - y0 + 1, nz = z1 - z0 + 1;
    const long long nb = (nx > 0 && ny > 0 && nz > 0) ? (long long)nx * ny * nz : 0;
    const S* f = reinterpret_cast<const S*>(a.f);
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (long long k = threadIdx.x; k < nb; k += blockDim.x) {
        const int x = x0 + (int)(k % nx), y = y0 + (int)((k / nx) % ny), z = z0 + (int)(k / ((long long)nx * ny));
        const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
        const uint8_t t = a.ntype[i];
        if (!is_active(t)) continue;
        if (t & HB_INSIDE) {
            if ((int)a.solid[i] == p) acc[6] += 1.0;
            continue;
        }
        if (t & HB_BULK) continue;  // every link of a bulk node ends on a fluid node
        for (int j = 1; j < Q; ++j) {
            const int xl = x + cx(j), yl = y + cy(j), zl = z + cz(j);
            const long long l = (long long)xl + (long long)a.X * ((long long)yl + (long long)a.Y * zl);
            const uint8_t tl = a.ntype[l];
            if (!(is_active(tl) && (tl & HB_INSIDE)) || (int)a.solid[l] != p) continue;
            double ux, uy, uz;
            mbb_velocity(a.parts, p, xl, yl, zl, ux, uy, uz);
            const double BBi = 6.0 * a.rho[i] * wgt(j) * (ux * cx(j) + uy * cy(j) + uz * cz(j));
            double fo = (double)P::load(f + (long long)opp(j) * a.N + i);
            if (P::DEV) fo += wgt(j);
            const double sc = 2.0 * ((fo + BBi) - 1.0 * wgt(j)) - BBi;
            const double Fx = sc * cx(j), Fy = sc * cy(j), Fz = sc * cz(j);
            const double rx = (double)xl - cxp, ry = (double)yl - cyp, rz = (double)zl - czp;
            acc[0] += Fx; acc[1] += Fy; acc[2] += Fz;
            acc[3] += ry * Fz - rz * Fy;
            acc[4] += rz * Fx - rx * Fz;
            acc[5] += rx * Fy - ry * Fx;
        }
    }
    for (int q = 0; q < 7; ++q) sh[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int q = 0; q < 7; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int q = 0; q < 3; ++q) {
            a.FH[(long long)q * E + p] = sh[q][0];
            a.MH[(long long)q * E + p] = sh[3 + q][0];
        }
        a.fvol[p] = sh[6][0];
    }
}

static MbbArgs mbb_args(hb_ctx* c, void* f) {
    MbbArgs m;
    m.X = c->X; m.Y = c->Y; m.Z = c->Z; m.N = c->N;
    m.ntype = c->ntype;
    m.solid = c->solid;
    m.f = f;
    m.rho = c->rho;
    const LBArgs la = lb_args(c, 0);
    m.parts = la.parts;
    m.pop = c->d.pop_list;
    m.npop = c->d.pop_cnt;
    m.pop_rho = c->d.pop_rho;
    m.claims = c->d.claim_list;
    m.nclaim = c->d.claim_cnt;
    m.FH = c->d.FH; m.MH = c->d.MH; m.fvol = c->d.fvol;
    return m;
}

// after the coupling masks of the step whose lattice update reads buffer `cur`; the
// lists live on the device, so the grids cover their capacity and exit early
void launch_mbb_nodes(hb_ctx* c, int cur) {
    MbbArgs m = mbb_args(c, cur ? c->fB : c->fA);
    const int B = 256;
    // the lists hold a few thousand entries per step: a fixed grid with grid-stride loops
    // (the launch shape does not depend on the device-side counts)
    const unsigned gp = 152 * 4;
    if (c->P.precision == HB_FP64) launch_pdl(k_mbb_refill_gs<PolF64>, gp, B, c->stream, m);
    else if (c->P.precision == HB_FP32) launch_pdl(k_mbb_refill_gs<PolF32>, gp, B, c->stream, m);
    else launch_pdl(k_mbb_refill_gs<PolF16>, gp, B, c->stream, m);
    launch_pdl(k_mbb_relink_gs, gp, B, c->stream, m, init_args(c), per_faces(c), c->lmask);
}

void launch_mbb_force(hb_ctx* c, int cur) {
    MbbArgs m = mbb_args(c, cur ? c->fA : c->fB);  // the buffer the step just wrote
    if (c->P.precision == HB_FP64) k_mbb_force<PolF64><<<c->d.E, 256, 0, c->stream>>>(m);
    else if (c->P.precision == HB_FP32) k_mbb_force<PolF32><<<c->d.E, 256, 0, c->stream>>>(m);
    else k_mbb_force<PolF16><<<c->d.E, 256, 0, c->stream>>>(m);
}

}  // namespace hb
