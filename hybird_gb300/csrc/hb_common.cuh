// hb_common.cuh -- shared device definitions of the sm_103a time-step library.
//
// Data layout in HBM (one context, one GPU):
//   node byte  ntype[N]      : type code (node.h:75-86) | HB_INSIDE (particle flag) |
//                              HB_BULK (all 18 links lead to active nodes)
//   solid[N]   uint32        : particle index for inside nodes, wall/object index for walls
//   fA/fB      S[19*N]       : populations, structure-of-arrays f[j*N+i], ping-pong
//   rho[N], u[3N], hf[3N], mass[N] : FP64 node macros, written where a later phase
//                              (free surface, coupling, downloads) reads them
//   visc[N]    T             : persistent viscosity, only with Bingham/Smagorinsky
//   dv[3N]     T             : direct-forcing term per inside-particle node
// Index i = x + X*(y + Y*z), exactly the reference's (LB.cpp:2314-2370).
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/hybird_gpu.h"

#define HB_TYPE_MASK 0x0F
#define HB_INSIDE 0x10
#define HB_BULK 0x20
#define HB_MIRROR 0x80  // the lattice kernels write this node's FP64 velocity (curved walls read it)
#define HB_PWRAP 0x40   // some link of this node crosses a periodic face

namespace hb {

constexpr int Q = 19;
constexpr int MAX_WALLS = 6;
constexpr int NBR_CAP = 48;      // candidate neighbours kept per particle unless hb_params.cap_neighbors says otherwise
constexpr int OBJ_CAP = 16;      // objects in range kept per particle
constexpr int STATUS_WORDS = 8;  // device status words (numeric, capacity, wait, ...)
constexpr int PARTIAL_CAP = 4096;  // per-block partials of grid-wide reductions (>= any grid used)
constexpr int MAX_MULTI = 64;      // DEM substeps per cycle (their maxima use the last partial slots)
// fixed-point scale of the element force/torque/volume sums of the reduced-precision
// lattice kernels: 64-bit integer sums are exact and order-free, so the atomics that
// build them give the same bits on every run
constexpr double HACC_SCALE = 274877906944.0;  // 2^38
constexpr double HACC_INV = 1.0 / 274877906944.0;

// D3Q19 velocity set in the reference's order O,x,y,z,xy,yz,zx (lattice.h:36-60)
__host__ __device__ constexpr int cx(int j) {
    return j == 1 || j == 7 || j == 10 || j == 15 || j == 17 ? 1
         : (j == 2 || j == 8 || j == 9 || j == 16 || j == 18 ? -1 : 0);
}
__host__ __device__ constexpr int cy(int j) {
    return j == 3 || j == 7 || j == 9 || j == 11 || j == 14 ? 1
         : (j == 4 || j == 8 || j == 10 || j == 12 || j == 13 ? -1 : 0);
}
__host__ __device__ constexpr int cz(int j) {
    return j == 5 || j == 11 || j == 13 || j == 15 || j == 18 ? 1
         : (j == 6 || j == 12 || j == 14 || j == 16 || j == 17 ? -1 : 0);
}
__host__ __device__ constexpr int opp(int j) { return j == 0 ? 0 : ((j & 1) ? j + 1 : j - 1); }
__host__ __device__ constexpr double wgt(int j) {
    return j == 0 ? 12.0 / 36.0 : (j <= 6 ? 2.0 / 36.0 : 1.0 / 36.0);
}

__device__ __forceinline__ bool is_active(uint8_t t) {
    const uint8_t c = t & HB_TYPE_MASK;
    return c == HB_T_FLUID || c == HB_T_INTERFACE;
}
// an active node the lattice updates: with moving bounce-back (mbb) the nodes inside
// particles are solid
__device__ __forceinline__ bool is_fluid(uint8_t t, int mbb) { return is_active(t) && !(mbb && (t & HB_INSIDE)); }

// ---- population load/store cache policy ----------------------------------------------
// HB_CACHE_HINT 1: streaming (evict-first) loads and stores; 0: default caching.
#ifndef HB_CACHE_HINT
#define HB_CACHE_HINT 0
#endif
#if HB_CACHE_HINT
#define HB_LD(p) __ldcs(p)
#define HB_ST(p, v) __stcs(p, v)
#else
#define HB_LD(p) (*(p))
#define HB_ST(p, v) (*(p) = (v))
#endif

// ---- storage precision policies ------------------------------------------------------
// FP64: full populations in double, compute in double (the reference's arithmetic).
// FP32: deviations g = f - w*rho0 in float, compute in float.
// FP16S: deviations scaled by 2^SHIFT in half, compute in float.
struct PolF64 {
    using S = double;
    using T = double;
    static constexpr bool DEV = false;
    __device__ static __forceinline__ T load(const S* p) { return HB_LD(p); }
    __device__ static __forceinline__ void store(S* p, T v) { HB_ST(p, v); }
    __device__ static __forceinline__ S enc(T v) { return v; }
    __device__ static __forceinline__ S enc_store(T v) { return v; }
};
struct PolF32 {
    using S = float;
    using T = float;
    static constexpr bool DEV = true;
    __device__ static __forceinline__ T load(const S* p) { return HB_LD(p); }
    __device__ static __forceinline__ void store(S* p, T v) { HB_ST(p, v); }
    __device__ static __forceinline__ S enc(T v) { return v; }
    __device__ static __forceinline__ S enc_store(T v) { return v; }
    // the stored value itself (units of UNIT per deviation): the lattice kernel computes on
    // these, so FP16 storage needs no scaling per load and store
    static constexpr float UNIT = 1.0f;
    static constexpr float INVU = 1.0f;
    __device__ static __forceinline__ T load_raw(const S* p) { return HB_LD(p); }
    __device__ static __forceinline__ S enc_raw(T v) { return v; }
    __device__ static __forceinline__ void store_raw(S* p, T v) { HB_ST(p, v); }
};
struct PolF16 {
    using S = __half;
    using T = float;
    static constexpr bool DEV = true;
    static constexpr float SCALE = 32768.0f;
    static constexpr float INV = 1.0f / 32768.0f;
    __device__ static __forceinline__ T load(const S* p) {
        const unsigned short b = HB_LD(reinterpret_cast<const unsigned short*>(p));
        return __half2float(__ushort_as_half(b)) * INV;
    }
    __device__ static __forceinline__ void store(S* p, T v) {
        HB_ST(reinterpret_cast<unsigned short*>(p), __half_as_ushort(__float2half_rn(v * SCALE)));
    }
    __device__ static __forceinline__ S enc_store(T v) { return __float2half_rn(v * SCALE); }
    static constexpr float UNIT = SCALE;
    static constexpr float INVU = INV;
    __device__ static __forceinline__ T load_raw(const S* p) {
        return __half2float(__ushort_as_half(HB_LD(reinterpret_cast<const unsigned short*>(p))));
    }
    __device__ static __forceinline__ S enc_raw(T v) { return __float2half_rn(v); }
    __device__ static __forceinline__ void store_raw(S* p, T v) {
        HB_ST(reinterpret_cast<unsigned short*>(p), __half_as_ushort(__float2half_rn(v)));
    }
};

// ---- device-side views of the context ----------------------------------------------
struct Particles {          // DEM elements as the coupling sees them (FP64)
    int count;
    const double* x0;       // [3*E] particle centre (corrected)
    const double* x1;       // [3*E] velocity
    const double* w;        // [3*E] wGlobal
    const double* radius;   // [E]
    const float* pf;        // [12*(E+gcap)] FP32 copy per particle: centre, velocity, wGlobal, pad
    // per-particle path (periodic faces, multi-sphere elements), else null: element of
    // every particle and the centre its lever arm is taken from (stride pstride)
    const int* pkey;
    const double* pcen;
    long long pstride;
};

struct LBArgs {
    int X, Y, Z;
    long long N;
    int per[6];             // face periodic flags (boundary code 4), x-,x+,y-,y+,z-,z+
    uint8_t* ntype;
    uint32_t* solid;
    const void* fin;        // populations after the previous streaming (read)
    void* fout;             // populations after this step's streaming (written)
    const int* mode;       // bit0: write all node macros (downloads)
    double* rho;
    double* u;              // [3N]
    double* hf;             // [3N]
    double* mass;
    void* visc;             // T[N] when viscosity is persistent
    void* dv;               // T[3N] direct-forcing term of inside nodes (FP64 kernel)
    unsigned long long* hacc;  // [7E] fixed-point F, M, fluid volume per element (FP32/FP16 kernels)
    const unsigned long long* lmask;  // [N] non-bulk active node: bits 0-18 links that need the general
                                      // push, bits 32-50 links ending on a static wall
    const double* F;        // device body force [3] (zero when forceFieldSolve = 0)
    const float* Ff;        // the same force in FP32 for the reduced-precision kernels
    int ne[Q];              // index offset of link j for nodes whose links do not wrap
    int jn[Q];              // j * N: start of direction j in a population array
    int so[Q];              // j * N + ne[j]: push target of direction j from node 0
    float init_visc_f, trt_magic_f, plastic_visc_f, yield_stress_f, turb_const_f;
    double init_visc;
    int collision;
    double trt_magic;
    int visc_model;         // bit0 Bingham, bit1 Smagorinsky
    double plastic_visc, yield_stress, turb_const;
    int free_surface;
    int couple;             // direct forcing of the nodes inside particles
    int mbb;                // moving bounce-back: nodes inside particles are solid
    Particles parts;
    int* status;            // [STATUS_WORDS]
    double* wall_part;      // [grid * (MAX_WALLS*3 + 1)] per-CTA moving-wall partials
    int nwalls;
};

inline int ceil_div(long long a, int b) { return (int)((a + b - 1) / b); }

__device__ __forceinline__ void flag_status(int* status, int word) { atomicOr(status + word, 1); }

// Programmatic dependent launch for chains of short kernels: a kernel launched with
// launch_pdl may be scheduled while its predecessor in the stream still runs, so its
// launch latency hides behind that kernel's tail.  Every such kernel starts with
// pdl_enter(): it waits until the predecessor grid has completed and its memory is
// visible (griddepcontrol.wait) before any access, then lets its own successor be
// scheduled.  In a kernel launched normally both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace hb
