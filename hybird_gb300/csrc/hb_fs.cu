// hb_fs.cu -- free-surface step (LB::latticeBoltzmannFreeSurfaceStep, LB.cpp:235-245,
// 1492-1804) as full-grid passes over the node byte.
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
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

enum : uint8_t { FS_FILLED = 1, FS_EMPTIED = 2, FS_NEW_A = 4, FS_NEW_B = 8 };
constexpr int FS_PARTS = 4;  // ledger partials: K3, K4, K5, K6

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
    int blocks;
};

__device__ __forceinline__ long long fs_link(const FsArgs& a, long long i, int j) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
    return (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
}
__device__ __forceinline__ bool interior(const FsArgs& a, long long i) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    return x > 0 && y > 0 && z > 0 && x < a.X - 1 && y < a.Y - 1 && z < a.Z - 1;
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
    __shared__ double sh[256];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.part[(long long)k * a.blocks + blockIdx.x] = sh[0];
    __syncthreads();
}

// K1 updateMass (LB.cpp:1492-1590): newMass = mass + sum_j a_j (f[opp j] - fs[j])
template <class P>
__global__ void k_fs_mass(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    if (code_of(a, i) != HB_T_INTERFACE) return;
    const bool first = *a.first != 0;
    const double mi = a.mass[i];
    double dm = 0.0;
    for (int j = 1; j < Q; ++j) {
        const long long l = fs_link(a, i, j);
        const uint8_t t = code_of(a, l);
        double av = 0.0;
        if (t == HB_T_INTERFACE) av = 0.5 * (a.mass[l] + mi);
        else if (t == HB_T_FLUID) av = 1.0;
        else if (t == HB_T_DYNWALL) av = 1.0 * mi;
        else continue;  // gas, static wall: averageMass 0
        const double fin = fval<P>(a, opp(j), i);
        double fs;
        if (first) fs = fval<P>(a, j, i);  // f = fs = f_eq at initialisation
        else if (t == HB_T_DYNWALL) {
            const double uw = a.u[l] * cx(j) + a.u[a.N + l] * cy(j) + a.u[2 * a.N + l] * cz(j);
            fs = fin + 6.0 * a.rho[i] * wgt(j) * uw;  // f[opp j] = fs[j] - BBi
        } else fs = fval<P>(a, j, l);              // pushed to the active neighbour
        dm += 1.0 * av * (fin - fs);
    }
    a.mass2[i] = mi + dm;
}

// K2 findInterfaceMutants (LB.cpp:1620-1650)
__global__ void k_fs_classify(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const uint8_t t = a.ntype[i];
    uint8_t fl = 0;
    if ((t & HB_TYPE_MASK) == HB_T_FLUID) a.mass[i] = a.rho[i];  // fluid mass = n (LB.cpp:1582-1585)
    if ((t & HB_TYPE_MASK) == HB_T_INTERFACE) {
        const double m = a.mass2[i];
        a.mass[i] = m;
        if (m > a.rho[i]) {
            fl = FS_FILLED;
            a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_FLUID;
        } else if (m < 0.0) {
            fl = FS_EMPTIED;
            a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_GAS;
        }
    }
    a.flag[i] = fl;
}

// K3 smoothenInterface, gas neighbours of filled cells (LB.cpp:1657-1677)
template <class P>
__global__ void k_fs_new_from_filled(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double contrib = 0.0;
    if (i < a.N && code_of(a, i) == HB_T_GAS && interior(a, i)) {
        long long parent = -1;
        for (int k = 1; k < Q; ++k) {  // filled cell m with link d[m][j] == i
            const long long m = fs_link(a, i, k);
            if (!(a.flag[m] & FS_FILLED) || !interior(a, m)) continue;
            if (fs_link(a, m, opp(k)) != i) continue;
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
            contrib = -0.01 * 1.0;
        }
    }
    block_ledger(a, 0, contrib);
}

// K4 smoothenInterface, fluid neighbours of emptied cells (LB.cpp:1679-1700)
__global__ void k_fs_new_from_emptied(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double contrib = 0.0;
    if (i < a.N && code_of(a, i) == HB_T_FLUID && interior(a, i)) {
        bool hit = false;
        for (int k = 1; k < Q && !hit; ++k) {
            const long long m = fs_link(a, i, k);
            if (!(a.flag[m] & FS_EMPTIED) || !interior(a, m)) continue;
            if (fs_link(a, m, opp(k)) == i) hit = true;
        }
        if (hit) {
            const double n = a.rho[i];
            a.mass[i] = 0.99 * n;
            contrib = 0.01 * n;
            a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_INTERFACE;
            a.flag[i] |= FS_NEW_B;
        }
    }
    block_ledger(a, 1, contrib);
}

// K5 updateMutants (LB.cpp:1703-1742) and removeIsolated, first pass (LB.cpp:1749-1769)
__global__ void k_fs_mutants_to_fluid(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double contrib = 0.0;
    if (i < a.N) {
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
                if (code_of(a, fs_link(a, i, j)) == HB_T_GAS) gas = true;
            if (!gas) {
                contrib += a.mass[i] - a.rho[i];
                a.mass[i] = a.rho[i];
                a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_FLUID;
            }
        }
    }
    block_ledger(a, 2, contrib);
}

// K6 removeIsolated, second pass (LB.cpp:1771-1793)
__global__ void k_fs_isolated_gas(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double contrib = 0.0;
    int count = 0;
    if (i < a.N && code_of(a, i) == HB_T_INTERFACE) {
        bool fluid = false;
        for (int j = 1; j < Q && !fluid; ++j)
            if (code_of(a, fs_link(a, i, j)) == HB_T_FLUID) fluid = true;
        if (!fluid) {
            contrib = a.mass[i];
            a.ntype[i] = (a.ntype[i] & ~HB_TYPE_MASK) | HB_T_GAS;
        } else {
            count = 1;
        }
    }
    block_ledger(a, 3, contrib);
    __shared__ int shc[256];
    shc[threadIdx.x] = count;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) shc[threadIdx.x] += shc[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.cnt_part[blockIdx.x] = shc[0];
}

// ledger total (fixed order over kernels and blocks) and interface count
__global__ void k_fs_ledger(FsArgs a) {
    __shared__ double shs[256];
    __shared__ long long shc[256];
    double s = 0.0;
    long long c = 0;
    for (int b = threadIdx.x; b < a.blocks; b += blockDim.x) {
        for (int k = 0; k < FS_PARTS; ++k) s += a.part[(long long)k * a.blocks + b];
        c += a.cnt_part[b];
    }
    shs[threadIdx.x] = s;
    shc[threadIdx.x] = c;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            shs[threadIdx.x] += shs[threadIdx.x + k];
            shc[threadIdx.x] += shc[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.scal[0] = shs[0];
        a.scal[1] = (double)shc[0];
        *a.first = 0;
    }
}

// K7 redistributeMass (LB.cpp:1796-1804)
__global__ void k_fs_redistribute(FsArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N || code_of(a, i) != HB_T_INTERFACE) return;
    a.mass[i] += a.scal[0] / a.scal[1];
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
    a.blocks = ceil_div(c->N, 256);
    return a;
}

int fs_init(hb_ctx* c) {
    const long long N = c->N;
    const int blocks = ceil_div(N, 256);
    if (cudaMalloc(&c->fs_flag, N) != cudaSuccess || cudaMalloc(&c->fs_mass2, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&c->fs_part, sizeof(double) * FS_PARTS * blocks) != cudaSuccess ||
        cudaMalloc(&c->fs_cnt, sizeof(int) * blocks) != cudaSuccess ||
        cudaMalloc(&c->fs_scal, sizeof(double) * 2) != cudaSuccess ||
        cudaMalloc(&c->fs_first, sizeof(int)) != cudaSuccess)
        return HB_ERR_NOMEM;
    cudaMemset(c->fs_flag, 0, N);
    cudaMemset(c->fs_scal, 0, sizeof(double) * 2);
    const int one = 1;
    cudaMemcpy(c->fs_first, &one, sizeof(int), cudaMemcpyHostToDevice);
    return cudaGetLastError() == cudaSuccess ? HB_OK : HB_ERR_CUDA;
}

void launch_fs_step(hb_ctx* c, int cur) {
    FsArgs a = fs_args(c, cur);
    const int G = a.blocks, B = 256;
    cudaStream_t s = c->stream;
    if (c->P.precision == HB_FP64) k_fs_mass<PolF64><<<G, B, 0, s>>>(a);
    else if (c->P.precision == HB_FP32) k_fs_mass<PolF32><<<G, B, 0, s>>>(a);
    else k_fs_mass<PolF16><<<G, B, 0, s>>>(a);
    k_fs_classify<<<G, B, 0, s>>>(a);
    if (c->P.precision == HB_FP64) k_fs_new_from_filled<PolF64><<<G, B, 0, s>>>(a);
    else if (c->P.precision == HB_FP32) k_fs_new_from_filled<PolF32><<<G, B, 0, s>>>(a);
    else k_fs_new_from_filled<PolF16><<<G, B, 0, s>>>(a);
    k_fs_new_from_emptied<<<G, B, 0, s>>>(a);
    k_fs_mutants_to_fluid<<<G, B, 0, s>>>(a);
    k_fs_isolated_gas<<<G, B, 0, s>>>(a);
    k_fs_ledger<<<1, 256, 0, s>>>(a);
    k_fs_redistribute<<<G, B, 0, s>>>(a);
    launch_refresh_bulk(c);  // node types changed
}

}  // namespace hb
