// hb_adjoint.cu -- reverse-mode derivative of the single-phase lattice step with
// bounce-back, for the drag on fixed spheres (objects).
//
// Forward model, per step and active node (g = f - w*rho0, rho0 = 1):
//   collision   the pairwise TRT form of the FP32 lattice kernel with Guo forcing
//               (node.cpp:90-101, 158-184; BGK when w- = w+), body force F uniform;
//   streaming   push; link to an active node -> g_j(l) = h_j(i); static wall or
//               object -> g_opp(i) = h_j(i) (LB.cpp:1344-1356); moving wall ->
//               g_opp(i) = h_j(i) - 6 n w_j (u_w . c_j) (LB.cpp:1321-1341), where the
//               moving-wall nodes of the planes x = 0 and x = X-1 take the caller's inlet
//               field u_w = (u_in(y,z), 0, 0) and other moving walls keep their velocity.
// Objective: J = drag on all objects along one axis, measured in the last of T steps:
//   J = sum over (active i, j) whose link is an object node of 2 h_j(i) c_j,axis,
//   i.e. node::bounceBackForce (node.cpp:283-291) with BBi = 0 summed over the links.
//   Objects are the reference's fixed spheres turned into static wall nodes
//   (LB.cpp:535-550); the reference itself reports no force on them.
// Reverse: lambda^t = (dPhi/dg^t)^T lambda^{t+1} with lambda^{T-1} = dJ/dg^{T-1}.  The
// transpose of push streaming is a pull of lambda^{t+1}; the transpose of the local
// collision is, with mu the pulled adjoint of the 19 post-collision values,
//   lambda_k = (L^T mu)_k + A + c_k . B,
// L the (self-adjoint) relaxation of the pair halves and (A, B) the derivative of the
// moment-dependent part (equilibrium and Guo term) with respect to (rho, momentum).
// Parameter gradients are summed over all steps: dJ/dF, dJ/dw+ and dJ/dw- (combined on
// the host into dJ/dtau), and per moving-wall link of the x planes dJ/du_in.
// Memory: the state g is checkpointed every K steps in HBM during the forward pass; the
// reverse pass recomputes each segment into an in-HBM tape and walks it backwards.
// All sums are deterministic: fixed thread ownership and fixed-order block reductions.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {
namespace {

enum : uint8_t {
    K_ACT = 0,    // fluid (or interface) node
    K_WALL = 1,   // static wall that is not an object
    K_OBJ = 2,    // object node (static wall inside an object sphere)
    K_INLET = 3,  // moving wall on x = 0 or x = X-1: velocity (u_in(y,z), 0, 0)
    K_MOV = 4,    // other moving wall: velocity from the context's node velocity
    K_SKIP = 5,   // periodic layer: never the end of a link
    K_BAD = 6,    // node kind outside the single-phase model (gas, curved, slip)
    K_CODE = 0x07,
    K_BULK = 0x08 // active node whose 18 links reach active nodes without wrapping
};

constexpr int AMAXW = 8;  // warps per block at most (blockDim.x <= 256)
constexpr int NPART = 8;  // per-block partials: dF[3], G+, G-, J, 2 spare

struct Geom {
    int X, Y, Z;
    long long N;
    int per[6];
    int ne[Q];
    const uint8_t* kind;
    const double* uwall;  // [3N] context node velocities (moving walls other than inlets)
    int axis;
};

template <class R>
struct Coef {
    R wp, wm, ap, am;
    R F[3];
};

__device__ __forceinline__ int alink(const Geom& G, int x, int y, int z, int j) {
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && G.per[0]) xn = G.X - 2;
    else if (xn == G.X - 1 && G.per[1]) xn = 1;
    if (yn == 0 && G.per[2]) yn = G.Y - 2;
    else if (yn == G.Y - 1 && G.per[3]) yn = 1;
    if (zn == 0 && G.per[4]) zn = G.Z - 2;
    else if (zn == G.Z - 1 && G.per[5]) zn = 1;
    return xn + G.X * (yn + G.Y * zn);
}

// c_j . v and acc + c s with the zero components of c_j left out (compile-time j):
// without fast-math the compiler keeps every 0 * v product
template <class R>
__device__ __forceinline__ R cdotR(int j, R vx, R vy, R vz) {
    R r;
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
template <class R>
__device__ __forceinline__ R addc(R acc, int c, R s) { return c == 0 ? acc : (c > 0 ? acc + s : acc - s); }

template <class R>
struct Mac {
    R dn, n, inv, ux, uy, uz, usq, uF;
};

template <class R>
__device__ __forceinline__ void macros(const R* g, const Coef<R>& C, Mac<R>& M) {
    R dn = 0, mx = 0, my = 0, mz = 0;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        dn += g[j];
        if (cx(j)) mx += cx(j) > 0 ? g[j] : -g[j];
        if (cy(j)) my += cy(j) > 0 ? g[j] : -g[j];
        if (cz(j)) mz += cz(j) > 0 ? g[j] : -g[j];
    }
    M.dn = dn;
    M.n = R(1) + dn;
    M.inv = R(1) / M.n;
    M.ux = (mx + R(0.5) * C.F[0]) * M.inv;  // shiftVelocity (node.cpp:85-88)
    M.uy = (my + R(0.5) * C.F[1]) * M.inv;
    M.uz = (mz + R(0.5) * C.F[2]) * M.inv;
    M.usq = M.ux * M.ux + M.uy * M.uy + M.uz * M.uz;
    M.uF = M.ux * C.F[0] + M.uy * C.F[1] + M.uz * C.F[2];
}

// post-collision deviations h[19] (the FP32 lattice kernel's pairwise form)
template <class R>
__device__ __forceinline__ void collide(const R* g, const Mac<R>& M, const Coef<R>& C, R* h) {
    const R w0 = R(wgt(0));
    const R e0 = w0 * (M.dn + M.n * (R(-1.5) * M.usq));
    h[0] = g[0] - C.wp * (g[0] - e0) + C.ap * (w0 * (R(-3) * M.uF));
#pragma unroll
    for (int j = 1; j < Q; j += 2) {
        const int o = j + 1;
        const R w = R(wgt(j));
        const R vu = cdotR<R>(j, M.ux, M.uy, M.uz);
        const R cF = cdotR<R>(j, C.F[0], C.F[1], C.F[2]);
        const R ep = w * (M.dn + M.n * (R(4.5) * vu * vu - R(1.5) * M.usq));
        const R em = R(3) * w * M.n * vu;
        const R fp = R(0.5) * (g[j] + g[o]), fm = R(0.5) * (g[j] - g[o]);
        const R Fs = w * (R(9) * vu * cF - R(3) * M.uF), Fa = R(3) * w * cF;
        const R sym = fp - C.wp * (fp - ep) + C.ap * Fs;
        const R anti = fm - C.wm * (fm - em) + C.am * Fa;
        h[j] = sym + anti;
        h[o] = sym - anti;
    }
}

// Transpose of the local collision: mu[19] (adjoint of h) is replaced by lambda[19]
// (adjoint of g); Awall is the extra adjoint of rho from moving-wall links.  gr
// accumulates dF (3), d/dw+ and d/dw-.
template <class R>
__device__ __forceinline__ void adj_local(const R* g, R* mu, R Awall, const Mac<R>& M, const Coef<R>& C,
                                          R* gr) {
    const R n = M.n, ux = M.ux, uy = M.uy, uz = M.uz, usq = M.usq;
    const R Fx = C.F[0], Fy = C.F[1], Fz = C.F[2];
    R Adn = 0, Bx = 0, By = 0, Bz = 0;  // Phi_rho at fixed u, Phi_u
    {
        const R w0 = R(wgt(0));
        const R m0 = mu[0];
        const R e0 = w0 * (M.dn + n * (R(-1.5) * usq));
        const R S0 = w0 * (R(-3) * M.uF);
        Adn += m0 * C.wp * w0 * (R(1) - R(1.5) * usq);
        const R k0 = m0 * R(-3) * w0;
        Bx += k0 * (C.wp * n * ux + C.ap * Fx);
        By += k0 * (C.wp * n * uy + C.ap * Fy);
        Bz += k0 * (C.wp * n * uz + C.ap * Fz);
        gr[0] += k0 * C.ap * ux;
        gr[1] += k0 * C.ap * uy;
        gr[2] += k0 * C.ap * uz;
        gr[3] += m0 * (-(g[0] - e0) - R(0.5) * S0);
        mu[0] = (R(1) - C.wp) * m0;
    }
#pragma unroll
    for (int j = 1; j < Q; j += 2) {
        const int o = j + 1;
        const R w = R(wgt(j));
        const R vu = cdotR<R>(j, ux, uy, uz);
        const R cF = cdotR<R>(j, Fx, Fy, Fz);
        const R ep = w * (M.dn + n * (R(4.5) * vu * vu - R(1.5) * usq));
        const R em = R(3) * w * n * vu;
        const R fp = R(0.5) * (g[j] + g[o]), fm = R(0.5) * (g[j] - g[o]);
        const R Fs = w * (R(9) * vu * cF - R(3) * M.uF), Fa = R(3) * w * cF;
        const R s = mu[j] + mu[o], d = mu[j] - mu[o];
        Adn += s * C.wp * w * (R(1) + R(4.5) * vu * vu - R(1.5) * usq) + d * C.wm * R(3) * w * vu;
        // d/du of s (w+ e+ + a+ S+) + d (w- e-): c-direction and u-direction parts
        const R kc = s * (C.wp * w * n * R(9) * vu + C.ap * w * R(9) * cF) + d * C.wm * R(3) * w * n;
        const R ku = s * C.wp * w * n * R(-3);
        const R kF = s * C.ap * w * R(-3);
        Bx += addc<R>(ku * ux + kF * Fx, cx(j), kc);
        By += addc<R>(ku * uy + kF * Fy, cy(j), kc);
        Bz += addc<R>(ku * uz + kF * Fz, cz(j), kc);
        // direct dependence of S+ and S- on F
        const R gc = s * C.ap * w * R(9) * vu + d * C.am * R(3) * w;
        const R gu = s * C.ap * w * R(-3);
        gr[0] += addc<R>(gu * ux, cx(j), gc);
        gr[1] += addc<R>(gu * uy, cy(j), gc);
        gr[2] += addc<R>(gu * uz, cz(j), gc);
        gr[3] += s * (-(fp - ep) - R(0.5) * Fs);
        gr[4] += d * (-(fm - em) - R(0.5) * Fa);
        const R ls = R(0.5) * (R(1) - C.wp) * s, ld = R(0.5) * (R(1) - C.wm) * d;
        mu[j] = ls + ld;
        mu[o] = ls - ld;
    }
    // chain through u = (m + F/2)/n: du/dm = 1/n, du/drho = -u/n, du/dF = 1/(2n)
    const R inv = M.inv;
    const R bx = Bx * inv, by = By * inv, bz = Bz * inv;
    const R A = Adn - (bx * ux + by * uy + bz * uz) + Awall;
    gr[0] += R(0.5) * bx;
    gr[1] += R(0.5) * by;
    gr[2] += R(0.5) * bz;
#pragma unroll
    for (int k = 0; k < Q; ++k) mu[k] += addc<R>(addc<R>(addc<R>(A, cx(k), bx), cy(k), by), cz(k), bz);
}

// Deterministic block sum of nv per-thread values into part[blk*NPART + off ...]: warp
// shuffles in R, the warps combined in R in warp order by one thread per value, added to
// the block's FP64 slot.  (Combining them in FP64 on one thread cost a serial chain of
// FP64 additions per block on this part's narrow FP64 pipe.)
template <class R>
__device__ __forceinline__ void block_accumulate(R* v, int nv, int off, double* part) {
    __shared__ R sh[NPART][AMAXW];
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, wid = tid >> 5;
    for (int k = 0; k < nv; ++k) {
        R x = v[k];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) x += __shfl_down_sync(0xffffffffu, x, s);
        if (lane == 0) sh[k][wid] = x;
    }
    __syncthreads();
    if (tid < nv) {
        const int nw = (blockDim.x * blockDim.y + 31) >> 5;
        const long long blk = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        R t = R(0);
        for (int w = 0; w < nw; ++w) t += sh[tid][w];
        part[blk * NPART + off + tid] += (double)t;
    }
}

// ---- kernels ------------------------------------------------------------------------

__global__ void k_adj_kind(Geom G, const uint8_t* ntype, const double* ox, const double* orad, int O, uint8_t* kind) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= G.N) return;
    const int x = (int)(i % G.X), y = (int)((i / G.X) % G.Y), z = (int)(i / ((long long)G.X * G.Y));
    const uint8_t t = ntype[i] & HB_TYPE_MASK;
    uint8_t k = K_BAD;
    if (t == HB_T_FLUID || t == HB_T_INTERFACE) k = K_ACT;
    else if (t == HB_T_PERIODIC) k = K_SKIP;
    else if (t == HB_T_STATWALL) {
        k = K_WALL;
        for (int o = 0; o < O; ++o) {  // the object test of the lattice initialisation
            const double dx = x - ox[o], dy = y - ox[O + o], dz = z - ox[2 * O + o];
            if (dx * dx + dy * dy + dz * dz < orad[o] * orad[o]) { k = K_OBJ; break; }
        }
    } else if (t == HB_T_DYNWALL) k = (x == 0 || x == G.X - 1) ? K_INLET : K_MOV;
    kind[i] = k;
}

// BULK bit and link check (status[0] set when an active node links to a kind outside
// the model)
__global__ void k_adj_bulk(Geom G, uint8_t* kind, int* bad) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1, z = blockIdx.z + 1;
    if (x >= G.X) return;
    const int i = x + G.X * (y + G.Y * z);
    if ((kind[i] & K_CODE) != K_ACT) return;
    bool bulk = true;
    for (int j = 1; j < Q; ++j) {
        const int l = alink(G, x, y, z, j);
        const int kl = kind[l] & K_CODE;
        if (kl == K_SKIP || kl == K_BAD) atomicOr(bad, 1);
        if (kl != K_ACT || l != i + G.ne[j]) bulk = false;
    }
    if (bulk) kind[i] = K_ACT | K_BULK;
}

// state of the context (any storage precision) -> deviations in R
template <class P, class R>
__global__ void k_adj_load(Geom G, const typename P::S* f, R* g) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= G.N) return;
    const bool act = (G.kind[i] & K_CODE) == K_ACT;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        R v = R(0);
        if (act) {
            const auto fv = P::load(f + j * G.N + i);
            v = P::DEV ? R(fv) : R(double(fv) - wgt(j));
        }
        g[j * G.N + i] = v;
    }
}

template <class R>
__device__ __forceinline__ R wall_cu(const Geom& G, const R* uin, int l, int j) {
    const int code = G.kind[l] & K_CODE;
    if (code == K_INLET) {
        const int yl = (l / G.X) % G.Y, zl = l / (G.X * G.Y);
        return R(cx(j)) * uin[yl + G.Y * zl];
    }
    return R(G.uwall[l] * cx(j) + G.uwall[G.N + l] * cy(j) + G.uwall[2 * G.N + l] * cz(j));
}

template <class R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 5 : 1) k_adj_fwd(Geom G, Coef<R> C, const R* __restrict__ gin,
                                                 R* __restrict__ gout, const R* __restrict__ uin) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1, z = blockIdx.z * blockDim.y + threadIdx.y + 1;
    if (x >= G.X || z > G.Z - 2) return;
    const int N = (int)G.N;
    const int i = x + G.X * (y + G.Y * z);
    const uint8_t k = G.kind[i];
    if ((k & K_CODE) != K_ACT) return;
    R g[Q], h[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) g[j] = gin[j * N + i];
    Mac<R> M;
    macros(g, C, M);
    collide(g, M, C, h);
    gout[i] = h[0];
    if (k & K_BULK) {
#pragma unroll
        for (int j = 1; j < Q; ++j) gout[j * N + i + G.ne[j]] = h[j];
        return;
    }
#pragma unroll
    for (int j = 1; j < Q; ++j) {
        const int l = alink(G, x, y, z, j);
        const int kl = G.kind[l] & K_CODE;
        const int o = opp(j);
        if (kl == K_ACT) gout[j * N + l] = h[j];
        else if (kl == K_WALL || kl == K_OBJ) gout[o * N + i] = h[j];
        else gout[o * N + i] = h[j] - R(6) * M.n * R(wgt(j)) * wall_cu(G, uin, l, j);
    }
}

// Terminal step: lambda^{T-1} = (dD/dg)^T with D the object drag of the collision of
// g^{T-1}; also adds the drag itself and dD/dtheta to the block partials.
template <class R>
__global__ void __launch_bounds__(256) k_adj_terminal(Geom G, Coef<R> C, const R* __restrict__ gin,
                                                      R* __restrict__ lout, double* part) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1, z = blockIdx.z + 1;
    const int N = (int)G.N;
    R gr[6] = {0, 0, 0, 0, 0, 0};
    if (x < G.X) {
        const int i = x + G.X * (y + G.Y * z);
        const uint8_t k = G.kind[i];
        if ((k & K_CODE) == K_ACT) {
            R g[Q], mu[Q];
            bool any = false;
            mu[0] = R(0);
#pragma unroll
            for (int j = 1; j < Q; ++j) {
                mu[j] = R(0);
                if (!(k & K_BULK) && (G.kind[alink(G, x, y, z, j)] & K_CODE) == K_OBJ) {
                    const int c = G.axis == 0 ? cx(j) : (G.axis == 1 ? cy(j) : cz(j));
                    mu[j] = R(2 * c);
                    any = true;
                }
            }
            if (any) {
#pragma unroll
                for (int j = 0; j < Q; ++j) g[j] = gin[j * N + i];
                Mac<R> M;
                macros(g, C, M);
                R h[Q];
                collide(g, M, C, h);
                R Jl = 0;
#pragma unroll
                for (int j = 1; j < Q; ++j) Jl += mu[j] * h[j];
                gr[5] = Jl;
                adj_local(g, mu, R(0), M, C, gr);
            }
#pragma unroll
            for (int j = 0; j < Q; ++j) lout[j * N + i] = mu[j];
        }
    }
    block_accumulate(gr, 6, 0, part);
}

// One reverse step: lambda^t from lambda^{t+1} (pulled) and g^t (recomputed forward).
// FP32: at most 64 registers (a few spilled) measured 2 % faster than 80.
template <class R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 1) k_adj_step(Geom G, Coef<R> C, const R* __restrict__ gin,
                                                  const R* __restrict__ lin, R* __restrict__ lout,
                                                  const R* __restrict__ uin, double* __restrict__ acc,
                                                  double* part) {
    // blockDim.y z rows per block: the block's partial sums (a barrier and an FP64
    // addition per value) are paid once for all of them
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y + 1, z = blockIdx.z * blockDim.y + threadIdx.y + 1;
    const int N = (int)G.N;
    R gr[5] = {0, 0, 0, 0, 0};
    if (x < G.X && z <= G.Z - 2) {
        const int i = x + G.X * (y + G.Y * z);
        const uint8_t k = G.kind[i];
        if ((k & K_CODE) == K_ACT) {
            R g[Q], mu[Q];
#pragma unroll
            for (int j = 0; j < Q; ++j) g[j] = gin[j * N + i];
            Mac<R> M;
            macros(g, C, M);
            R Awall = 0;
            mu[0] = lin[i];
            if (k & K_BULK) {
#pragma unroll
                for (int j = 1; j < Q; ++j) mu[j] = lin[j * N + i + G.ne[j]];
            } else {
#pragma unroll
                for (int j = 1; j < Q; ++j) {
                    const int l = alink(G, x, y, z, j);
                    const int kl = G.kind[l] & K_CODE;
                    const int o = opp(j);
                    if (kl == K_ACT) {
                        mu[j] = lin[j * N + l];
                    } else {
                        mu[j] = lin[o * N + i];
                        if (kl == K_INLET || kl == K_MOV) {
                            const R w6 = R(-6) * R(wgt(j)) * mu[j];
                            Awall += w6 * wall_cu(G, uin, l, j);
                            if (kl == K_INLET) {  // dJ/du_in of this link, owned by node i
                                const int side = (l % G.X) == 0 ? 0 : 1;
                                acc[((long long)(side * Q + j)) * (G.Y * G.Z) + y + G.Y * z] +=
                                    (double)(w6 * M.n * R(cx(j)));
                            }
                        }
                    }
                }
            }
            adj_local(g, mu, Awall, M, C, gr);
#pragma unroll
            for (int j = 0; j < Q; ++j) lout[j * N + i] = mu[j];
        }
    }
    block_accumulate(gr, 5, 0, part);
}

// fixed-order sum of the block partials -> out[NPART]
__global__ void k_adj_final(const double* part, long long nblk, double* out) {
    __shared__ double sh[NPART][256];
    for (int k = 0; k < NPART; ++k) {
        double t = 0.0;
        for (long long b = threadIdx.x; b < nblk; b += blockDim.x) t += part[b * NPART + k];
        sh[k][threadIdx.x] = t;
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < NPART; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < NPART; ++k) out[k] = sh[k][0];
}

// dJ/du_in(y,z): sum over the links that end on the inlet nodes (0,y,z) and (X-1,y,z),
// gathered from the link owners' accumulators in a fixed (side, direction) order
__global__ void k_adj_inlet(Geom G, const double* acc, double* grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.Y * G.Z) return;
    const int yl = q % G.Y, zl = q / G.Y;
    double t = 0.0;
    for (int side = 0; side < 2; ++side) {
        const int xl = side == 0 ? 0 : G.X - 1;
        const int l = xl + G.X * (yl + G.Y * zl);
        if ((G.kind[l] & K_CODE) != K_INLET) continue;
        for (int j = 1; j < Q; ++j) {
            int xi = xl - cx(j), yi = yl - cy(j), zi = zl - cz(j);
            if (xi < 0 || xi >= G.X) continue;
            if (yi == G.Y - 1 && G.per[2]) yi = 1;  // inverse of the periodic remap
            else if (yi == 0 && G.per[3]) yi = G.Y - 2;
            if (zi == G.Z - 1 && G.per[4]) zi = 1;
            else if (zi == 0 && G.per[5]) zi = G.Z - 2;
            if (yi < 1 || yi > G.Y - 2 || zi < 1 || zi > G.Z - 2 || xi < 1 || xi > G.X - 2) continue;
            const int i = xi + G.X * (yi + G.Y * zi);
            if ((G.kind[i] & K_CODE) != K_ACT || alink(G, xi, yi, zi, j) != l) continue;
            t += acc[((long long)(side * Q + j)) * (G.Y * G.Z) + yi + G.Y * zi];
        }
    }
    grad[q] = t;
}

}  // namespace

struct hb_adj {
    int prec = -1, K = 0, C = 0, slots = 0;
    long long N = 0;
    size_t s = 0;
    char* ck = nullptr;
    char* tape = nullptr;
    char* lam[2] = {nullptr, nullptr};
    uint8_t* kind = nullptr;
    double* acc = nullptr;
    double* part = nullptr;
    double* out = nullptr;
    double* grad = nullptr;
    void* uin = nullptr;
    int* bad = nullptr;
    long long nblk = 0;
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    float ms_fwd = 0.f, ms_rev = 0.f;
    long long fwd_steps = 0, rev_steps = 0;
};

static void adj_release(hb_adj* a) {
    void* ptrs[] = {a->ck, a->tape, a->lam[0], a->lam[1], a->kind, a->acc, a->part, a->out, a->grad, a->uin, a->bad};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto& ev : a->e)
        if (ev) cudaEventDestroy(ev);
    *a = hb_adj();
}

void adjoint_free(hb_ctx* c) {
    if (!c->adj) return;
    adj_release(c->adj);
    delete c->adj;
    c->adj = nullptr;
}

namespace {

struct Launch {
    dim3 grid, block;
    long long nblk;
};

Launch node_launch(const hb_ctx* c) {
    Launch L;
    const int bx = c->X <= 256 ? ((c->X + 31) / 32) * 32 : 128;
    L.block = dim3((unsigned)bx);
    L.grid = dim3((unsigned)ceil_div(c->X, bx), (unsigned)(c->Y - 2), (unsigned)(c->Z - 2));
    L.nblk = (long long)L.grid.x * L.grid.y * L.grid.z;
    return L;
}

int fail(std::string& err, int code, const char* msg) {
    err = msg;
    return code;
}

#define ACK(call)                                                                      \
    do {                                                                               \
        cudaError_t _e = (call);                                                       \
        if (_e != cudaSuccess) {                                                       \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);                  \
            return HB_ERR_CUDA;                                                        \
        }                                                                              \
    } while (0)

int adj_alloc(hb_ctx* c, hb_adj* a, int prec, int K, int C, std::string& err) {
    const long long N = c->N;
    const size_t s = prec == HB_FP64 ? 8 : 4;
    const int slots = K < 3 ? 3 : K;
    if (a->prec == prec && a->K == K && a->C == C && a->N == N) return HB_OK;
    adj_release(a);
    const size_t S19 = (size_t)Q * N * s;
    size_t fr = 0, tot = 0;
    ACK(cudaMemGetInfo(&fr, &tot));
    const size_t need = S19 * ((size_t)C + slots + 2) + (size_t)N + (size_t)2 * Q * c->Y * c->Z * 8;
    if (need + (size_t)(256u << 20) > fr) {
        char m[256];
        snprintf(m, sizeof(m), "adjoint needs %.2f GB of device memory (checkpoints + tape), %.2f GB free",
                 need / 1e9, fr / 1e9);
        return fail(err, HB_ERR_NOMEM, m);
    }
    Launch L = node_launch(c);
    auto al = [&](void** p, size_t bytes) -> int {
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            err = "cudaMalloc failed in the adjoint";
            return HB_ERR_NOMEM;
        }
        return HB_OK;
    };
    int rc;
    if ((rc = al((void**)&a->ck, S19 * C)) || (rc = al((void**)&a->tape, S19 * slots)) ||
        (rc = al((void**)&a->lam[0], S19)) || (rc = al((void**)&a->lam[1], S19)) ||
        (rc = al((void**)&a->kind, (size_t)N)) || (rc = al((void**)&a->acc, (size_t)2 * Q * c->Y * c->Z * 8)) ||
        (rc = al((void**)&a->part, (size_t)L.nblk * NPART * 8)) || (rc = al((void**)&a->out, NPART * 8)) ||
        (rc = al((void**)&a->grad, (size_t)c->Y * c->Z * 8)) || (rc = al(&a->uin, (size_t)c->Y * c->Z * 8)) ||
        (rc = al((void**)&a->bad, sizeof(int)))) {
        adj_release(a);
        return rc;
    }
    ACK(cudaMemset(a->lam[0], 0, S19));
    ACK(cudaMemset(a->lam[1], 0, S19));
    ACK(cudaMemset(a->tape, 0, S19 * slots));
    for (auto& ev : a->e) ACK(cudaEventCreate(&ev));
    a->prec = prec;
    a->K = K;
    a->C = C;
    a->N = N;
    a->s = s;
    a->slots = slots;
    a->nblk = L.nblk;
    return HB_OK;
}

template <class R>
int adj_run(hb_ctx* c, hb_adj* a, const hb_adjoint_cfg* cfg, bool reverse, Geom G, double* J, double* dF,
            double* dtau, double* duin, std::string& err) {
    cudaStream_t st = c->stream;
    const long long N = c->N;
    const size_t S19 = (size_t)Q * N * sizeof(R);
    const int T = cfg->steps, K = cfg->checkpoint_every, Cn = a->C;
    Launch L = node_launch(c);

    // relaxation rates of the forward model and their derivatives with respect to tau
    const double tau = cfg->tau;
    const double wp = 1.0 / tau;
    const bool trt = c->P.collision == HB_TRT;
    const double lam = c->P.trt_magic;
    const double wm = trt ? 1.0 / (lam / (tau - 0.5) + 0.5) : wp;
    const double dwp = -1.0 / (tau * tau);
    const double dwm = trt ? wm * wm * lam / ((tau - 0.5) * (tau - 0.5)) : dwp;
    Coef<R> C;
    C.wp = R(wp);
    C.wm = R(wm);
    C.ap = R(1.0 - 0.5 * wp);
    C.am = R(1.0 - 0.5 * wm);
    for (int k = 0; k < 3; ++k) C.F[k] = R(cfg->body_force[k]);

    // inlet field in R
    {
        std::vector<R> h((size_t)c->Y * c->Z, R(0));
        if (cfg->inlet_velocity)
            for (size_t q = 0; q < h.size(); ++q) h[q] = R(cfg->inlet_velocity[q]);
        ACK(cudaMemcpyAsync(a->uin, h.data(), h.size() * sizeof(R), cudaMemcpyHostToDevice, st));
        ACK(cudaStreamSynchronize(st));  // h is a stack buffer
    }
    const R* uin = reinterpret_cast<const R*>(a->uin);
    ACK(cudaMemsetAsync(a->acc, 0, (size_t)2 * Q * c->Y * c->Z * 8, st));
    ACK(cudaMemsetAsync(a->part, 0, (size_t)a->nblk * NPART * 8, st));

    auto state = [&](int cidx, int s) -> R* {
        return reinterpret_cast<R*>(s == 0 ? a->ck + (size_t)cidx * S19 : a->tape + (size_t)s * S19);
    };
    auto lamb = [&](int p) { return reinterpret_cast<R*>(a->lam[p]); };

    ACK(cudaEventRecord(a->e[0], st));
    // g^0 from the context's current state
    {
        const int B = 256, Gd = ceil_div(N, B);
        R* g0 = state(0, 0);
        if (c->P.precision == HB_FP64)
            k_adj_load<PolF64, R><<<Gd, B, 0, st>>>(G, (const double*)(c->cur ? c->fB : c->fA), g0);
        else if (c->P.precision == HB_FP32)
            k_adj_load<PolF32, R><<<Gd, B, 0, st>>>(G, (const float*)(c->cur ? c->fB : c->fA), g0);
        else
            k_adj_load<PolF16, R><<<Gd, B, 0, st>>>(G, (const __half*)(c->cur ? c->fB : c->fA), g0);
    }
    // forward blocks: as many z rows as fit in 256 threads
    const unsigned frows = L.block.x >= 256 ? 1u : 256u / L.block.x;
    const dim3 FB(L.block.x, frows), FG(L.grid.x, L.grid.y, (unsigned)ceil_div(L.grid.z, (int)frows));
    // forward pass: g^0 .. g^{T-1}, checkpoints at multiples of K
    R* cur = state(0, 0);
    for (int t = 0; t + 1 <= T - 1; ++t) {
        R* out = ((t + 1) % K == 0) ? state((t + 1) / K, 0) : state(0, 1 + (t & 1));
        k_adj_fwd<R><<<FG, FB, 0, st>>>(G, C, cur, out, uin);
        cur = out;
    }
    a->fwd_steps = T - 1;
    a->rev_steps = 0;
    if (!reverse) k_adj_terminal<R><<<L.grid, L.block, 0, st>>>(G, C, cur, lamb(0), a->part);
    ACK(cudaGetLastError());
    ACK(cudaEventRecord(a->e[1], st));
    if (reverse) {
        int p = 0;
        // reverse-step blocks: as many z rows as fit in 256 threads
        const unsigned rows = L.block.x >= 256 ? 1u : 256u / L.block.x;
        const dim3 LSb(L.block.x, rows), LSg(L.grid.x, L.grid.y, (unsigned)ceil_div(L.grid.z, (int)rows));
        for (int ci = Cn - 1; ci >= 0; --ci) {
            const int t0 = ci * K;
            const int t1 = (t0 + K < T ? t0 + K : T) - 1;
            for (int s = 0; s < t1 - t0; ++s)
                k_adj_fwd<R><<<FG, FB, 0, st>>>(G, C, state(ci, s), state(ci, s + 1), uin);
            a->fwd_steps += t1 - t0;
            for (int t = t1; t >= t0; --t) {
                R* g = state(ci, t - t0);
                if (t == T - 1) {
                    k_adj_terminal<R><<<L.grid, L.block, 0, st>>>(G, C, g, lamb(p), a->part);
                } else {
                    k_adj_step<R><<<LSg, LSb, 0, st>>>(G, C, g, lamb(p), lamb(1 - p), uin, a->acc, a->part);
                    p ^= 1;
                    a->rev_steps += 1;
                }
            }
        }
        ACK(cudaGetLastError());
        k_adj_inlet<<<ceil_div((long long)c->Y * c->Z, 128), 128, 0, st>>>(G, a->acc, a->grad);
    }
    k_adj_final<<<1, 256, 0, st>>>(a->part, a->nblk, a->out);
    ACK(cudaGetLastError());
    ACK(cudaEventRecord(a->e[2], st));
    double out[NPART];
    ACK(cudaMemcpyAsync(out, a->out, sizeof(out), cudaMemcpyDeviceToHost, st));
    if (reverse && duin)
        ACK(cudaMemcpyAsync(duin, a->grad, sizeof(double) * c->Y * c->Z, cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    ACK(cudaEventElapsedTime(&a->ms_fwd, a->e[0], a->e[1]));
    ACK(cudaEventElapsedTime(&a->ms_rev, a->e[1], a->e[2]));
    if (J) *J = out[5];
    if (reverse) {
        if (dF)
            for (int k = 0; k < 3; ++k) dF[k] = out[k];
        if (dtau) *dtau = out[3] * dwp + out[4] * dwm;
    }
    if (!std::isfinite(out[5])) return fail(err, HB_ERR_NUMERIC, "adjoint: drag is not finite");
    return HB_OK;
}

}  // namespace

int adjoint_run(hb_ctx* c, const hb_adjoint_cfg* cfg, bool reverse, double* J, double* dF, double* dtau,
                double* duin, std::string& err) {
    if (!c->initialized) return fail(err, HB_ERR_STATE, "hb_init has not run");
    if (!cfg) return fail(err, HB_ERR_ARG, "cfg is NULL");
    if (cfg->steps < 1) return fail(err, HB_ERR_ARG, "adjoint: steps must be >= 1");
    if (cfg->checkpoint_every < 1) return fail(err, HB_ERR_ARG, "adjoint: checkpoint_every must be >= 1");
    if (cfg->precision != HB_FP64 && cfg->precision != HB_FP32)
        return fail(err, HB_ERR_ARG, "adjoint: precision must be HB_FP64 or HB_FP32");
    if (!(cfg->tau > 0.5)) return fail(err, HB_ERR_ARG, "adjoint: tau must be > 0.5");
    if (cfg->drag_axis < 0 || cfg->drag_axis > 2) return fail(err, HB_ERR_ARG, "adjoint: drag_axis must be 0, 1 or 2");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(cfg->body_force[k])) return fail(err, HB_ERR_ARG, "adjoint: body force is not finite");
    if (c->P.free_surface || c->P.non_newtonian || c->P.turbulence)
        return fail(err, HB_ERR_UNSUPPORTED,
                    "adjoint: single-phase Newtonian lattices only (no free surface, Bingham or Smagorinsky)");
    if (c->d.E > 0)
        return fail(err, HB_ERR_UNSUPPORTED, "adjoint: moving particles are not part of the model; give fixed spheres as objects");
    if ((long long)Q * c->N >= (1LL << 31)) return fail(err, HB_ERR_UNSUPPORTED, "adjoint: lattice too large for 32-bit indices");
    if (!c->adj) c->adj = new hb_adj();
    hb_adj* a = c->adj;
    const int C = (cfg->steps - 1) / cfg->checkpoint_every + 1;
    int rc = adj_alloc(c, a, cfg->precision, cfg->checkpoint_every, C, err);
    if (rc) return rc;

    Geom G;
    G.X = c->X; G.Y = c->Y; G.Z = c->Z; G.N = c->N;
    for (int f = 0; f < 6; ++f) G.per[f] = c->P.boundary[f] == HB_T_PERIODIC;
    for (int j = 0; j < Q; ++j) G.ne[j] = cx(j) + c->X * (cy(j) + c->Y * cz(j));
    G.kind = a->kind;
    G.uwall = c->u;
    G.axis = cfg->drag_axis;
    cudaStream_t st = c->stream;
    {
        const int B = 256, Gd = ceil_div(c->N, B);
        k_adj_kind<<<Gd, B, 0, st>>>(G, c->ntype, c->d.obj_x0, c->d.obj_r, c->d.O, a->kind);
        Launch L = node_launch(c);
        ACK(cudaMemsetAsync(a->bad, 0, sizeof(int), st));
        k_adj_bulk<<<L.grid, L.block, 0, st>>>(G, a->kind, a->bad);
        int bad = 0;
        ACK(cudaMemcpyAsync(&bad, a->bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        if (bad) return fail(err, HB_ERR_UNSUPPORTED, "adjoint: an active node links to a node kind outside the model");
    }
    if (cfg->precision == HB_FP64) return adj_run<double>(c, a, cfg, reverse, G, J, dF, dtau, duin, err);
    return adj_run<float>(c, a, cfg, reverse, G, J, dF, dtau, duin, err);
}

int adjoint_timing(hb_ctx* c, float* ms_forward, float* ms_reverse, int64_t* fwd_steps, int64_t* rev_steps) {
    if (!c->adj) return HB_ERR_STATE;
    if (ms_forward) *ms_forward = c->adj->ms_fwd;
    if (ms_reverse) *ms_reverse = c->adj->ms_rev;
    if (fwd_steps) *fwd_steps = c->adj->fwd_steps;
    if (rev_steps) *rev_steps = c->adj->rev_steps;
    return HB_OK;
}

}  // namespace hb
