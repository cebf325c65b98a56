// hb_lb32.cu -- the reduced-precision fused collide+stream kernel (FP32 deviations or
// scaled FP16 deviations in HBM, FP32 arithmetic), compiled with FMA contraction.
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

// ---- reduced-precision kernel (FP32 / FP16 storage, FP32 compute) ---------------------
// Populations are deviations g = f - w (rho0 = 1).  The collision is written on the
// symmetric / antisymmetric parts of each direction pair (j, opp j):
//   g'_j   = sym + anti,   g'_opp = sym - anti,
//   sym  = fp - w+ (fp - ep) + (1 - w+/2) Fs,   anti = fm - w- (fm - em) + (1 - w-/2) Fa
// with fp, fm (ep, em; Fs, Fa) the halves of g_j +/- g_opp (of the equilibrium and of the
// Guo term).  BGK is the case w- = w+ = 1/tau: then g'_j = g_j + w (geq_j - g_j) + (1 - w/2)
// F_j, which is node::solveCollision + node::addForce (node.cpp:158-184).
// 32-bit indices; nodes whose links neither wrap nor touch a non-active node stream with
// fixed offsets ne[j].  (Measured on GB300: the scattered push stores cost no more than
// aligned or gathered ones; this kernel is bound by its instruction count.)

__device__ __forceinline__ int link32c(const LBArgs& a, int x, int y, int z, int kx, int ky, int kz) {
    int xn = x + kx, yn = y + ky, zn = z + kz;
    if (xn == 0 && a.per[0]) xn = a.X - 2;
    else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2;
    else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2;
    else if (zn == a.Z - 1 && a.per[5]) zn = 1;
    return xn + a.X * (yn + a.Y * zn);
}
__device__ __forceinline__ int link32(const LBArgs& a, int x, int y, int z, int j) {
    return link32c(a, x, y, z, cx(j), cy(j), cz(j));
}

// c_j . v with the zero components of c_j left out: without fast-math the compiler keeps
// every 0 * v product, so the sums are spelled out per direction (all branches fold)
__device__ __forceinline__ float cdot(int j, float vx, float vy, float vz) {
    float r;
    if (cx(j) != 0) {
        r = cx(j) > 0 ? vx : -vx;
        if (cy(j) != 0) r = cy(j) > 0 ? r + vy : r - vy;
        if (cz(j) != 0) r = cz(j) > 0 ? r + vz : r - vz;
    } else if (cy(j) != 0) {
        r = cy(j) > 0 ? vy : -vy;
        if (cz(j) != 0) r = cz(j) > 0 ? r + vz : r - vz;
    } else {
        r = cz(j) > 0 ? vz : -vz;
    }
    return r;
}

// v * 2^38 rounded to a 64-bit integer, from 32-bit conversions only (a 64-bit float to
// integer conversion issues on the narrow FP64 pipe of this part): a = |v| * 2^6 splits
// into floor(a) (the high word) and the exact fraction times 2^32 (the low word,
// < 2^32); the sign is applied to the 64-bit result.
__device__ __forceinline__ unsigned long long to_fixed(float v) {
    const float a = fabsf(v) * 64.0f;
    const float h = floorf(a);
    const unsigned long long m =
        ((unsigned long long)__float2uint_rn(h) << 32) + __float2uint_rn((a - h) * 4294967296.0f);
    return v < 0.0f ? 0ull - m : m;
}

// One post-collision population of a node with non-trivial links, the pull rules of
// LB.cpp:1231-1356 seen from the sending node.  (A form with selected target index and
// value, keeping the lanes of a warp converged, measured slower on GB300 than this
// branch chain.)
template <class P>
__device__ __forceinline__ void push_general(const LBArgs& a, typename P::S* fout, int x, int y, int z, int i,
                                             int j, float g, float n, float ux, float uy, float uz, float usq) {
    const int l = link32(a, x, y, z, j);
    const uint8_t lc = a.ntype[l] & HB_TYPE_MASK;
    const int o = opp(j);
    const int N = (int)a.N;
    if (lc == HB_T_FLUID || lc == HB_T_INTERFACE) {
        P::store_raw(fout + j * N + l, g);
    } else if (lc == HB_T_STATWALL || lc == HB_T_SLIPSTAT || lc == HB_T_SLIPDYN || lc == HB_T_CURVED) {
        // slip and curved walls: completed after the kernel (hb_slip.cu, hb_curved.cu)
        P::store_raw(fout + o * N + i, g);
    } else if (lc == HB_T_GAS) {
        const float vu = cdot(j, ux, uy, uz);
        const float w = float(wgt(j));
        P::store_raw(fout + o * N + i, -g + (w * P::UNIT) * (9.0f * vu * vu - 3.0f * usq));
    } else if (lc == HB_T_DYNWALL) {
        const float uw = float(a.u[l] * cx(j) + a.u[a.N + l] * cy(j) + a.u[2 * a.N + l] * cz(j));
        P::store_raw(fout + o * N + i, g - (6.0f * P::UNIT) * n * float(wgt(j)) * uw);
    } else {
        flag_status(a.status, 1);
    }
}

// Direction components of a link index known only at run time: 2-bit fields c + 1.
__host__ __device__ constexpr unsigned long long dir_bits(int k) {
    unsigned long long r = 0;
    for (int j = 0; j < Q; ++j)
        r |= (unsigned long long)((k == 0 ? cx(j) : (k == 1 ? cy(j) : cz(j))) + 1) << (2 * j);
    return r;
}
__device__ __forceinline__ int dir_rt(int k, int j) {
    constexpr unsigned long long B[3] = {dir_bits(0), dir_bits(1), dir_bits(2)};
    return (int)((B[k] >> (2 * j)) & 3ull) - 1;
}
// push_general of the moving-bounce-back kernel, out of line with the link index j
// (1..18) as a run-time value.  Next to particle surfaces most warps take the general
// push for several links; 18 inlined copies of this body (one per unrolled link) made
// the kernel instruction-fetch bound (no_instructions 51 % of the stall samples, local
// spills at 56 registers).  The arithmetic is push_general's, plus the particle links:
// BBi = 6 n w_j (u . c_j) with u the particle's velocity at the solid node, from its
// FP32 record (centre, velocity, spin); no link wraps in this mode.  The link's momentum
// exchange (2 (fs_j - w_j) - BBi) c_j (g = fs_j - w_j) and its moment about the element
// centre go to the node's sums mv for its first particle *mkey, or straight to another
// particle's fixed-point sums.
template <class P>
__device__ __forceinline__ void push_link_mbb(const LBArgs& a, int x, int y, int z, int i, int j, float g,
                                              float n, float* mv, int& mkey) {
    typename P::S* fout = reinterpret_cast<typename P::S*>(a.fout);
    const int kx = dir_rt(0, j), ky = dir_rt(1, j), kz = dir_rt(2, j);
    const int l = i + kx + a.X * (ky + a.Y * kz);  // no link wraps in this mode
    const uint8_t tl = a.ntype[l];
    const uint8_t lc = tl & HB_TYPE_MASK;
    const int o = (j & 1) ? j + 1 : j - 1;
    const int N = (int)a.N;
    const float w = j <= 6 ? float(wgt(1)) : float(wgt(7));
    const float fkx = (float)kx, fky = (float)ky, fkz = (float)kz;
    if ((tl & HB_INSIDE) && (lc == HB_T_FLUID || lc == HB_T_INTERFACE)) {
        const int pl = (int)a.solid[l];
        const float4* pf4 = reinterpret_cast<const float4*>(a.parts.pf) + 3 * (size_t)pl;
        const float4 q0 = pf4[0], q1 = pf4[1], q2 = pf4[2];
        const float rx = float(x + kx) - q0.x, ry = float(y + ky) - q0.y, rz = float(z + kz) - q0.z;
        const float wx = q1.z, wy = q1.w, wz = q2.x;
        const float vx = q0.w + (wy * rz - wz * ry), vy = q1.x + (wz * rx - wx * rz), vz = q1.y + (wx * ry - wy * rx);
        const float BBi = 6.0f * n * w * fmaf(fkz, vz, fmaf(fky, vy, fkx * vx));
        P::store_raw(fout + o * N + i, g - P::UNIT * BBi);
        const float sc = (2.0f * g - P::UNIT * BBi) * P::INVU;
        const float fx = fkx * sc, fy = fky * sc, fz = fkz * sc;
        const float v6[6] = {fx, fy, fz, ry * fz - rz * fy, rz * fx - rx * fz, rx * fy - ry * fx};
        if (mkey < 0) mkey = pl;
        if (pl == mkey) {
#pragma unroll
            for (int k = 0; k < 6; ++k) mv[k] += v6[k];
        } else {  // a second particle next to this node (rare)
            const int E = a.parts.count;
#pragma unroll
            for (int k = 0; k < 6; ++k) atomicAdd(a.hacc + (long long)k * E + pl, to_fixed(v6[k]));
        }
    } else if (lc == HB_T_FLUID || lc == HB_T_INTERFACE) {
        P::store_raw(fout + j * N + l, g);
    } else if (lc == HB_T_STATWALL || lc == HB_T_SLIPSTAT || lc == HB_T_SLIPDYN || lc == HB_T_CURVED) {
        P::store_raw(fout + o * N + i, g);
    } else if (lc == HB_T_DYNWALL) {
        const float uw = float(a.u[l] * kx + a.u[a.N + l] * ky + a.u[2 * a.N + l] * kz);
        P::store_raw(fout + o * N + i, g - (6.0f * P::UNIT) * n * w * uw);
    } else {  // gas links do not occur: no free surface in this mode
        flag_status(a.status, 1);
    }
}

// FP64 node fields (read by the free surface, the wall force and downloads) are written
// by separate non-inlined stores: inlined, their float -> double conversions would be
// executed for every node and occupy the narrow FP64 pipe.
__device__ __noinline__ void write_rho(double* rho, int i, float n) { rho[i] = (double)n; }
__device__ __noinline__ void write_u_hf(double* u, double* hf, long long N, int i, float ux, float uy, float uz,
                                        float hx, float hy, float hz) {
    u[i] = (double)ux; u[N + i] = (double)uy; u[2 * N + i] = (double)uz;
    hf[i] = (double)hx; hf[N + i] = (double)hy; hf[2 * N + i] = (double)hz;
}

// Element sums of the coupling (LB.cpp:1853-1918) folded into the lattice step: the
// nodes of one particle form runs of consecutive lanes along x; a segmented suffix sum
// over each run (fixed shuffle pattern) leaves the run total in its first lane, which
// adds it to the element's 64-bit fixed-point accumulators.  Integer sums do not depend
// on the order of the atomics, so the result is reproducible bit for bit.
__device__ __forceinline__ void element_sums_warp(unsigned long long* hacc, int E, int key, float* v) {
    const unsigned full = 0xffffffffu;
    if (!__any_sync(full, key >= 0)) return;
    const int lane = threadIdx.x & 31;
    const int knext = __shfl_down_sync(full, key, 1);
    const int kprev = __shfl_up_sync(full, key, 1);
    const unsigned ends = __ballot_sync(full, lane == 31 || knext != key);
    const int tail = lane + __ffs(ends >> lane) - 1;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const float o = __shfl_down_sync(full, v[k], off);
            if (lane + off <= tail) v[k] += o;
        }
    }
    if (key >= 0 && (lane == 0 || kprev != key)) {
#pragma unroll
        for (int k = 0; k < 7; ++k) atomicAdd(hacc + (long long)k * E + key, to_fixed(v[k]));
    }
}

// The update of one node from its 19 post-streaming deviations f: moments, coupling,
// collision, push.  Every lane of a warp calls it (act false for lanes without an active
// node), because the element sums use full-warp shuffles.
template <class P, bool MBB>
__device__ __forceinline__ void lb_node(const LBArgs& a, int x, int y, int z, int i, uint8_t t, bool act,
                                        float* f, int p, float4 q0, float4 q1, float4 q2, float* mv, int& mkey) {
    using S = typename P::S;
    const int N = (int)a.N;
    S* fout = reinterpret_cast<S*>(a.fout);
    const int mode = *a.mode;
    const uint8_t code = t & HB_TYPE_MASK;

    // f holds the stored values (units of P::UNIT); the sums scale exactly by INVU (a power
    // of two), so they equal the sums of the deviations bit for bit
    float dn = 0.0f, mx = 0.0f, my = 0.0f, mz = 0.0f;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        dn += f[j];
        if (cx(j)) mx += cx(j) > 0 ? f[j] : -f[j];
        if (cy(j)) my += cy(j) > 0 ? f[j] : -f[j];
        if (cz(j)) mz += cz(j) > 0 ? f[j] : -f[j];
    }
    dn *= P::INVU; mx *= P::INVU; my *= P::INVU; mz *= P::INVU;
    const float n = 1.0f + dn;
    const float inv = 1.0f / n;
    float ux = mx * inv, uy = my * inv, uz = mz * inv;
    if (!(n > 0.0f) || ux != ux || uy != uy || uz != uz) flag_status(a.status, 0);

    float hx = 0.0f, hy = 0.0f, hz = 0.0f;
    if (!MBB && a.couple) {
        int key = -1;
        float v[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (p >= 0) {  // LB.cpp:1863-1904 with FP32 particle copies

            const float rx = float(x) - q0.x, ry = float(y) - q0.y, rz = float(z) - q0.z;
            const float wx = q1.z, wy = q1.w, wz = q2.x;
            const float lvx = q0.w + (wy * rz - wz * ry);
            const float lvy = q1.x + (wz * rx - wx * rz);
            const float lvz = q1.y + (wx * ry - wy * rx);
            const float m = a.free_surface ? float(a.mass[i]) : 1.0f;
            const float lf = m * inv;
            const float dvx = lf * (ux - lvx), dvy = lf * (uy - lvy), dvz = lf * (uz - lvz);
            hx = -dvx; hy = -dvy; hz = -dvz;
            key = a.parts.pkey ? a.parts.pkey[p] : p;  // a particle sums into its element
            v[0] = dvx; v[1] = dvy; v[2] = dvz;  // element F, M, fluidVolume (LB.cpp:1893-1899)
            v[3] = ry * dvz - rz * dvy;
            v[4] = rz * dvx - rx * dvz;
            v[5] = rx * dvy - ry * dvx;
            v[6] = m;
        }
        element_sums_warp(a.hacc, a.parts.count, key, v);
    }
    // links that need the general push and links that end on a static wall (none for bulk
    // nodes: fixed push offsets)
    const bool fast = (t & (HB_BULK | HB_PWRAP)) == HB_BULK;
    const unsigned long long lm = fast ? 0ull : a.lmask[i];
    const uint32_t special = (uint32_t)lm, bb = (uint32_t)(lm >> 32);
    if (!act) return;
    const float Fx = a.Ff[0] + hx, Fy = a.Ff[1] + hy, Fz = a.Ff[2] + hz;
    ux += 0.5f * Fx * inv;  // shiftVelocity
    uy += 0.5f * Fy * inv;
    uz += 0.5f * Fz * inv;
    const float usq = ux * ux + uy * uy + uz * uz;
    const float uF = ux * Fx + uy * Fy + uz * Fz;

    float visc = a.init_visc_f;
    if (a.visc_model) {  // computeShearRate (node.cpp:103-145) on the symmetric parts
        float* vp = reinterpret_cast<float*>(a.visc);
        const float vold = vp[i];
        float pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
#pragma unroll
        for (int j = 1; j < Q; j += 2) {
            const int o = j + 1;
            const float vu = cdot(j, ux, uy, uz);
            const float w = float(wgt(j));
            const float ep = w * (dn + n * (4.5f * vu * vu - 1.5f * usq));
            const float d = (f[j] + f[o]) * P::INVU - 2.0f * ep;
            if (cx(j)) pxx += d;
            if (cy(j)) pyy += d;
            if (cz(j)) pzz += d;
            if (cx(j) * cy(j)) pxy += cx(j) * cy(j) > 0 ? d : -d;
            if (cx(j) * cz(j)) pxz += cx(j) * cz(j) > 0 ? d : -d;
            if (cy(j) * cz(j)) pyz += cy(j) * cz(j) > 0 ? d : -d;
        }
        const float tau = 0.5f + 3.0f * vold;
        const float sc = 1.5f / (tau * n);
        pxx *= sc; pyy *= sc; pzz *= sc; pxy *= sc; pxz *= sc; pyz *= sc;
        const float shear = sqrtf(0.5f * (pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz)));
        const float nuTurb = (a.visc_model & 2) ? a.turb_const_f * shear : 0.0f;
        const float nuApp = (a.visc_model & 1) ? a.plastic_visc_f + a.yield_stress_f / (n * 2.0f * shear) : vold;
        visc = fmaxf(float((0.501 - 0.5) / 3.0), fminf(float((1.8 - 0.5) / 3.0), nuApp + nuTurb));
        vp[i] = visc;
    }
    const float tp = 0.5f + 3.0f * visc;
    const float wp = 1.0f / tp;
    const float wm = a.collision == HB_TRT ? 1.0f / (a.trt_magic_f / (tp - 0.5f) + 0.5f) : wp;
    const float ap = 1.0f - 0.5f * wp, am = 1.0f - 0.5f * wm;

    const bool all = (mode & 1) != 0;
    if (all || a.free_surface || !(t & HB_BULK)) write_rho(a.rho, i, n);
    if (all || code == HB_T_INTERFACE || (t & HB_MIRROR)) write_u_hf(a.u, a.hf, a.N, i, ux, uy, uz, hx, hy, hz);

    // Pairwise collision with per-node coefficients for the two link weights (w = 1/18 on
    // the axes, 1/36 on the diagonals), S = g_j + g_o, D = g_j - g_o, base = dn - 1.5 n u^2:
    //   sym  = (1 - w+) S/2 + w+ w (base + 4.5 n vu^2) + a+ w (9 vu cF - 3 uF)
    //   anti = (1 - w-) D/2 + w- 3 w n vu + a- 3 w cF
    const float base = dn - 1.5f * n * usq;
    const float c1 = 0.5f * (1.0f - wp), c2 = 0.5f * (1.0f - wm);
    const float kb = wp * base - 3.0f * ap * uF;
    float K0[2], Kq[2], Kc[2], Lu[2], Lf[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const float w = q == 0 ? float(1.0 / 18.0) : float(1.0 / 36.0);
        // in units of P::UNIT, as f: the products scale exactly
        K0[q] = (w * kb) * P::UNIT;
        Kq[q] = (4.5f * wp * w * n) * P::UNIT;
        Kc[q] = (9.0f * ap * w) * P::UNIT;
        Lu[q] = (3.0f * wm * w * n) * P::UNIT;
        Lf[q] = (3.0f * am * w) * P::UNIT;
    }
    S* fo = fout + i;
    fo[0] = P::enc_raw(2.0f * c1 * f[0] + float(wgt(0)) * (kb * P::UNIT));  // rest population
#pragma unroll
    for (int j = 1; j < Q; j += 2) {  // post-collision values replace f in place
        const int o = j + 1;
        const int q = j <= 6 ? 0 : 1;
        const float vu = cdot(j, ux, uy, uz);
        const float cF = cdot(j, Fx, Fy, Fz);
        const float sym = fmaf(c1, f[j] + f[o], fmaf(Kq[q], vu * vu, fmaf(Kc[q] * vu, cF, K0[q])));
        const float anti = fmaf(c2, f[j] - f[o], fmaf(Lu[q], vu, Lf[q] * cF));
        f[j] = sym + anti;
        f[o] = sym - anti;
    }
    // Push.  The choice among the three forms is made per warp (all lanes that reach this
    // point), so that a warp of bulk nodes runs only plain stores and a warp next to a
    // static wall only the selected-offset stores; each form is exact for every lane.
    const unsigned warp = __activemask();
    if (__all_sync(warp, lm == 0ull)) {
#pragma unroll
        for (int j = 1; j < Q; ++j) fo[a.so[j]] = P::enc_raw(f[j]);
    } else if (__all_sync(warp, special == 0u)) {
        // a static (or slip) wall returns the population into the node's own opposite slot
#pragma unroll
        for (int j = 1; j < Q; ++j) fo[(bb & (1u << j)) ? opp(j) * N : a.so[j]] = P::enc_raw(f[j]);
    } else if constexpr (MBB) {
        // Next to particle surfaces most warps have general links, in different directions
        // per lane.  The plain and wall links are stored here; the general ones are staged
        // in shared memory and pushed by one loop over each lane's set bits (ascending j,
        // so the node's sums add in link order), so the lanes of a warp run that one body
        // together whatever their links.
        __shared__ float sf[Q - 1][128];
#pragma unroll
        for (int j = 1; j < Q; ++j) {
            if (special & (1u << j)) sf[j - 1][threadIdx.x] = f[j];
            else fo[(bb & (1u << j)) ? opp(j) * N : a.so[j]] = P::enc_raw(f[j]);
        }
        for (uint32_t s = special; s != 0u; s &= s - 1u) {
            const int j = __ffs(s) - 1;
            push_link_mbb<P>(a, x, y, z, i, j, sf[j - 1][threadIdx.x], n, mv, mkey);
        }
    } else {
#pragma unroll
        for (int j = 1; j < Q; ++j) {
            if (special & (1u << j)) push_general<P>(a, fout, x, y, z, i, j, f[j], n, ux, uy, uz, usq);
            else fo[(bb & (1u << j)) ? opp(j) * N : a.so[j]] = P::enc_raw(f[j]);
        }
    }
}

// One thread per node, populations loaded straight from HBM.  Nine blocks of 128 per SM
// (56 registers, no spills) measured faster than eight (64 registers) and ten (48, with
// spills).
// MBB: moving bounce-back (nodes inside particles are solid; their links bounce back
// with the particle's velocity and the momentum exchange builds the element sums); a
// separate instantiation, so the direct-forcing kernel keeps its instruction count.
template <class P, bool MBB>
__global__ void __launch_bounds__(128, 9) k_collide_stream_dev(LBArgs a) {
    using S = typename P::S;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1;
    const int z = blockIdx.z + 1;
    const int i = x + a.X * (y + a.Y * z);
    const S* fin = reinterpret_cast<const S*>(a.fin);
    // whole warps leave together so that the element sums can use full-warp shuffles;
    // lanes past the row end are inactive and marked bulk, so no link mask is read there
    const uint8_t t = x < a.X ? a.ntype[i] : (uint8_t)(HB_T_STATWALL | HB_BULK);
    const bool act = MBB ? is_fluid(t, 1) : is_active(t);
    const bool solidp = MBB && is_active(t) && (t & HB_INSIDE);  // counts its particle's volume
    if (!__any_sync(0xffffffffu, act || solidp)) return;
    // the particle index of a particle node is loaded ahead of the populations and its
    // particle's FP32 record right after them, so their latencies overlap the populations'
    // instead of following the moments (0.092 -> 0.082 ms per coupled 128^3 launch)
    const int p = (a.couple && act && (t & HB_INSIDE)) ? (int)a.solid[i] : -1;
    float f[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) f[j] = act ? P::load_raw(fin + a.jn[j] + i) : 0.0f;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0;
    if (p >= 0) {  // centre, velocity, spin
        const float4* pf4 = reinterpret_cast<const float4*>(a.parts.pf) + 3 * (size_t)p;
        q0 = pf4[0]; q1 = pf4[1]; q2 = pf4[2];
    }
    float mv[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int mkey = -1;
    if (MBB && solidp) {
        mkey = (int)a.solid[i];
        mv[6] = 1.0f;
    }
    lb_node<P, MBB>(a, x, y, z, i, t, act, f, p, q0, q1, q2, mv, mkey);
    if (MBB) element_sums_warp(a.hacc, a.parts.count, mkey, mv);  // every lane of the warp
}

void launch_lb_step_dev(hb_ctx* c, const LBArgs& a) {
    const int b2 = c->X <= 64 ? 64 : 128;
    dim3 g2((unsigned)ceil_div(c->X, b2), (unsigned)(c->Y - 2), (unsigned)(c->Z - 2));
    if (a.mbb) {
        if (c->P.precision == HB_FP32) k_collide_stream_dev<PolF32, true><<<g2, b2, 0, c->stream>>>(a);
        else k_collide_stream_dev<PolF16, true><<<g2, b2, 0, c->stream>>>(a);
    } else {
        if (c->P.precision == HB_FP32) k_collide_stream_dev<PolF32, false><<<g2, b2, 0, c->stream>>>(a);
        else k_collide_stream_dev<PolF16, false><<<g2, b2, 0, c->stream>>>(a);
    }
}

}  // namespace hb
