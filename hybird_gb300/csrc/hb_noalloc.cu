// hb_noalloc.cu -- moving-wall force reduction for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc: an application that reserves the device memory
// up front and hands each library a fixed budget (its own pool allocator owns the
// rest, so a cudaMalloc here would fail or break its accounting), and a host loop with
// a latency bound that cannot take the device-wide synchronisation a cudaMalloc or
// cudaFree may cause.  hb_wall_force_noalloc gives them the moving-wall momentum
// exchange (the reduction hb_download_walls reports) without any allocation: the
// per-CTA partial sums live in the file-scope device array below, of a fixed size,
// held by every GPU that loads this library until the process exits.
//
// Rules for callers:
//   * The first call on a device looks up the array's device address for that device
//     (cudaGetSymbolAddress) and keeps it; make that first call before any stream
//     capture.  A cudaDeviceReset unloads the array, so the kept address is stale
//     afterwards: do not call this entry point again in a process that reset the device.
//   * All calls share the array.  Every call rewrites all the partials it reads, so no
//     state carries over, but calls that overlap on the GPU (different streams, or
//     different host threads on one device) race on it and must be serialised by the
//     caller.
//   * Lattices above HB_NOALLOC_MAX_NODES nodes are rejected with HB_ERR_ARG.
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace {

constexpr int kParts = hb::MAX_WALLS * 3 + 1;  // per wall (Fx,Fy,Fz), plus the extra mass
constexpr int kBlocks = 1024;                  // fixed CTA count of the reduction
constexpr int kMaxDevices = 64;

// 19 x 1024 doubles = 152 KiB, shared by every call on a device
__device__ __align__(256) double g_wall_partials[kParts * kBlocks];

double* g_partials_addr[kMaxDevices] = {nullptr};

struct NoAllocArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    const double* f;
    const uint8_t* type;
    const uint32_t* solid;
    const double* rho;
    const double* u;
    const double* mass;
    double* partials;
    double* out;
};

// node bytes are compared on their type code: the library's internal flag bits
// (particle, bulk, wrap, mirror) may be set in a byte handed in from its own buffers
__device__ __forceinline__ bool act(uint8_t t) {
    const uint8_t c = t & HB_TYPE_MASK;
    return c == HB_T_FLUID || c == HB_T_INTERFACE;
}

// Same per-node arithmetic as the library's moving-wall reduction (LB.cpp:1321-1341),
// over a fixed grid that strides across the interior rows.
__global__ void __launch_bounds__(256) k_wall_noalloc(NoAllocArgs a) {
    __shared__ double sh[256];
    double acc[kParts];
#pragma unroll
    for (int k = 0; k < kParts; ++k) acc[k] = 0.0;
    const long long rows = (long long)(a.Y - 2) * (a.Z - 2);
    const long long items = rows * a.X;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
         it += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(it % a.X);
        const long long r = it / a.X;
        const int y = (int)(r % (a.Y - 2)) + 1, z = (int)(r / (a.Y - 2)) + 1;
        if (x < 1 || x > a.X - 2) continue;
        const long long i = (long long)x + (long long)a.X * ((long long)y + (long long)a.Y * z);
        if (!act(a.type[i])) continue;
        for (int j = 1; j < hb::Q; ++j) {
            int xn = x + hb::cx(j), yn = y + hb::cy(j), zn = z + hb::cz(j);
            if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
            if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
            if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
            const long long l = (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
            if ((a.type[l] & HB_TYPE_MASK) != HB_T_DYNWALL) continue;
            const double uw = a.u[l] * hb::cx(j) + a.u[a.N + l] * hb::cy(j) + a.u[2 * a.N + l] * hb::cz(j);
            const double BBi = 6.0 * a.rho[i] * hb::wgt(j) * uw;
            const double fsj = a.f[(long long)hb::opp(j) * a.N + i] + BBi;
            const double sc = (2.0 * (fsj - 1.0 * hb::wgt(j)) - BBi) * 1.0;
            const int w = (int)a.solid[l];
            // compile-time indices keep acc in registers (a runtime index would place it
            // in local memory)
#pragma unroll
            for (int ww = 0; ww < hb::MAX_WALLS; ++ww)
                if (ww == w) {
                    acc[3 * ww] += sc * hb::cx(j);
                    acc[3 * ww + 1] += sc * hb::cy(j);
                    acc[3 * ww + 2] += sc * hb::cz(j);
                }
            acc[hb::MAX_WALLS * 3] += BBi * a.mass[i];
        }
    }
    for (int k = 0; k < kParts; ++k) {  // fixed-order tree per partial
        sh[threadIdx.x] = acc[k];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) a.partials[(long long)k * kBlocks + blockIdx.x] = sh[0];
        __syncthreads();
    }
}

__global__ void k_wall_noalloc_final(const double* partials, double* out) {
    const int k = threadIdx.x;
    if (k >= kParts) return;
    double s = 0.0;
    for (int b = 0; b < kBlocks; ++b) s += partials[(long long)k * kBlocks + b];
    out[k] = s;
}

}  // namespace

extern "C" int hb_wall_force_noalloc(const double* f, const uint8_t* type, const uint32_t* solid,
                                     const double* rho, const double* u, const double* mass,
                                     const int32_t* lb_size, const int32_t* boundary, double* wall_force,
                                     void* stream) {
    if (!f || !type || !solid || !rho || !u || !mass || !lb_size || !boundary || !wall_force) return HB_ERR_ARG;
    for (int k = 0; k < 3; ++k)
        if (lb_size[k] < 3) return HB_ERR_ARG;
    const long long N = (long long)lb_size[0] * lb_size[1] * lb_size[2];
    if (N > HB_NOALLOC_MAX_NODES) return HB_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return HB_ERR_CUDA;
    if (!g_partials_addr[dev]) {  // once per device, with that device current
        double* p = nullptr;
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_wall_partials) != cudaSuccess || !p) return HB_ERR_CUDA;
        g_partials_addr[dev] = p;
    }
    NoAllocArgs a;
    a.X = lb_size[0]; a.Y = lb_size[1]; a.Z = lb_size[2]; a.N = N;
    for (int k = 0; k < 6; ++k) a.per[k] = boundary[k] == HB_T_PERIODIC;
    a.f = f; a.type = type; a.solid = solid; a.rho = rho; a.u = u; a.mass = mass;
    a.partials = g_partials_addr[dev];
    a.out = wall_force;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // launched through cudaLaunchKernel so that the status is this call's own: an error
    // another launch left pending on this thread is neither cleared nor reported here
    void* args1[] = {&a};
    if (cudaLaunchKernel(reinterpret_cast<const void*>(k_wall_noalloc), dim3(kBlocks), dim3(256), args1, 0, s) !=
        cudaSuccess)
        return HB_ERR_CUDA;
    double* partials = a.partials;
    void* args2[] = {&partials, &wall_force};
    if (cudaLaunchKernel(reinterpret_cast<const void*>(k_wall_noalloc_final), dim3(1), dim3(32), args2, 0, s) !=
        cudaSuccess)
        return HB_ERR_CUDA;
    return HB_OK;
}
