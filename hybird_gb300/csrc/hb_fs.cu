// hb_fs.cu -- free-surface step (LB::latticeBoltzmannFreeSurfaceStep, LB.cpp:235-245,
// 1492-1804) on compacted cell lists.
//
// The reference walks ordered lists (interface nodes sorted ascending, walked backwards;
// filled/emptied lists; appended new interface cells).  Every conversion rule it applies
// depends only on a node's own state and on neighbour types that the same pass does not
// change, so each rule becomes one parallel pass over a list:
//   K1 mass exchange of the interface cells (updateMass)              -> mass2
//   K2 classify the interface cells: mass > n filled -> fluid, mass < 0 emptied -> gas
//      (the conversion list); fluid cells take mass = n (one lean pass over the grid)
//   K3 gas cells next to a filled cell -> interface, initialised from the filled
//      neighbour with the LARGEST index (the reference visits filled cells in descending
//      order and the first visitor initialises the cell), surplus -= 0.01
//   K4 fluid cells next to an emptied cell -> interface, mass = 0.99 n, surplus += 0.01 n
//   K5 mutants (emptied not re-interfaced: surplus += mass; filled not re-interfaced:
//      surplus += mass - n, mass = n) and isolated interface without gas links -> fluid
//   K6 isolated interface without fluid links -> gas (surplus += mass); the others form
//      the next step's interface list
//   K7 surplus / count added to every interface cell (redistributeMass)
// K3 and K4 start from the conversion list and visit the cells' 18 neighbours; K5-K7 run
// over the interface cells (the list of the step's start minus the converted ones, plus
// the new ones).  The lists are unordered, so the FP64 surplus ledger is a 128-bit
// fixed-point sum (2^-100 resolution, integer atomics): its value does not depend on the
// order of the additions, and it differs from the reference's sequential FP64 sum at the
// rounding level only.
//
// Streamed populations: the reference's massStream(j) = f[opp j] - fs[j] needs the
// post-collision value fs[j] of the cell, which the push kernel delivered to the active
// neighbour in direction j (f[j] there), or which a moving wall turned into
// f[opp j] = fs[j] - BBi.  At the very first step fs is the initial equilibrium of the
// cell itself (node::initialize sets f = fs), and the first pass uses that.
#include <algorithm>
#include <cstddef>
#include <cstdio>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

enum : uint8_t { FS_FILLED = 1, FS_EMPTIED = 2, FS_NEW_A = 4, FS_NEW_B = 8 };
constexpr int FS_LIST_GRID = 152 * 4;  // blocks of 256 threads of the list passes

// Step state of the free surface in device memory (the fields from ccount on are zeroed
// at the start of every step).
struct FsCount {
    int first;       // 1 until the first free-surface step has run
    int valid;       // the current interface list holds the interface cells
    int sel;         // which of the two interface lists is current
    int changed;     // cells whose activity changed (gas <-> interface) in this step
    int icount[2];   // lengths of the two interface lists
    int ccount;      // filled and emptied cells of this step (the conversion list)
    int ncount;      // new interface cells of this step
    unsigned long long ledger[2];  // surplus of this step, 128-bit fixed point (low, high)
};
static_assert(sizeof(FsCount) <= 64, "the count block has 64 bytes");
constexpr double LEDGER_ONE = 1267650600228229401496703205376.0;  // 2^100

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
    uint8_t* flag;          // per-node conversion flags of this step (zero between steps)
    double* scal;           // [0] surplus [1] interface count [2] surplus / count
    const double* force;    // lbF as the free surface sees it (zeroed after the first step
                            // when forceFieldSolve = 0)
    FsCount* cnt;
    uint32_t* ilist;        // [2 * icap] the two interface lists (current, next)
    uint32_t* clist;        // [icap] filled and emptied cells of this step
    uint32_t* nlist;        // [icap] new interface cells of this step
    uint32_t* parent;       // [N] zero between steps: the filled parent (+1) of a new cell
    long long icap;         // capacity of each list (hb_params.cap_interface, default N)
    int* status;            // device status words (word 2, bit 8: interface list full)
};

struct Node {
    int x, y, z;
    long long i;
    bool ok;
};

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
__device__ __forceinline__ uint8_t code_of(const FsArgs& a, long long i) { return a.ntype[i] & HB_TYPE_MASK; }

template <class P>
__device__ __forceinline__ double fval(const FsArgs& a, int j, long long i) {
    double v = (double)P::load(reinterpret_cast<const typename P::S*>(a.f) + (long long)j * a.N + i);
    if (P::DEV) v += wgt(j);
    return v;
}

// ---- lists ------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t* cur_list(const FsArgs& a) { return a.ilist + (a.cnt->sel ? a.icap : 0); }
__device__ __forceinline__ uint32_t* next_list(const FsArgs& a) { return a.ilist + (a.cnt->sel ? 0 : a.icap); }
__device__ __forceinline__ int cur_count(const FsArgs& a) { return (int)min((long long)a.cnt->icount[a.cnt->sel], a.icap); }

// append `item` of the lanes with `take` to list[0 .. cap) at *count (warp ballot, one
// atomic per warp); a full list sets status word 2, bit 8
// The list passes deal 32-entry chunks of their list over the blocks first (chunk c to
// block c mod grid), so that a list of 10^4 cells reaches every SM instead of the first
// few dozen blocks; a whole warp takes each chunk, as the ballots of list_push need.
__device__ __forceinline__ int chunk_first() { return 32 * (blockIdx.x + gridDim.x * (threadIdx.x >> 5)) + (threadIdx.x & 31); }
__device__ __forceinline__ int chunk_stride() { return 32 * gridDim.x * (blockDim.x >> 5); }

__device__ __forceinline__ void list_push(const FsArgs& a, uint32_t* list, int* count, bool take, uint32_t item) {
    const unsigned warp = __activemask();
    const unsigned b = __ballot_sync(warp, take);
    if (!b) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(b) - 1;
    int base = 0;
    if (lane == leader) {
        base = atomicAdd(count, __popc(b));
        if (base + __popc(b) > a.icap) atomicOr(a.status + 2, 8);
    }
    base = __shfl_sync(warp, base, leader);
    const long long k = (long long)base + __popc(b & ((1u << lane) - 1u));
    if (take && k < a.icap) list[k] = item;
}

__device__ __forceinline__ Node node_at(const FsArgs& a, uint32_t iu) {
    const uint32_t X = (uint32_t)a.X, XY = (uint32_t)a.X * (uint32_t)a.Y;
    Node nd;
    nd.x = (int)(iu % X);
    nd.y = (int)((iu % XY) / X);
    nd.z = (int)(iu / XY);
    nd.i = (long long)iu;
    nd.ok = true;
    return nd;
}

// the surplus ledger: v * 2^100 rounded to the nearest 128-bit integer (ties to even),
// from the bits of v with integer instructions, added with two 64-bit atomics (the low
// word's carry goes into the high word with it).  Integer sums do not depend on the
// order of the additions.  |v| below 2^-54 rounds to 0; the total stays below 2^26.
__device__ void ledger_add(const FsArgs& a, double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FFu);
    if (e == 0) return;  // zero or subnormal
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int s = e - 1075 + 100;  // v 2^100 = m 2^s
    unsigned long long lo, hi;
    if (s >= 64) {
        lo = 0ull;
        hi = m << min(s - 64, 10);
    } else if (s > 0) {
        lo = m << s;
        hi = m >> (64 - s);
    } else if (s == 0) {
        lo = m;
        hi = 0ull;
    } else {
        const int k = -s;
        if (k > 54) return;
        const unsigned long long q = m >> k, rem = m & ((1ull << k) - 1ull), half = 1ull << (k - 1);
        lo = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
        hi = 0ull;
    }
    if (b >> 63) {  // two's complement of the 128-bit magnitude
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    const unsigned long long old = atomicAdd(&a.cnt->ledger[0], lo);
    atomicAdd(&a.cnt->ledger[1], hi + ((old + lo < old) ? 1ull : 0ull));
}

// K1 updateMass (LB.cpp:1492-1590): newMass = mass + sum_j a_j (f[opp j] - fs[j])
// The interface list is carried from step to step (K6 writes the next one); after an
// upload or a restore of the node types it is rebuilt here from the node bytes, by warp
// ballots (order within the list is irrelevant: each cell's mass exchange is independent
// of the others).
__global__ void __launch_bounds__(256) k_fs_ilist(FsArgs a) {
    pdl_enter();
    if (a.cnt->valid) return;
    uint32_t* list = cur_list(a);
    int* count = &a.cnt->icount[a.cnt->sel];
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n_up = (a.N + 31) / 32 * 32;  // whole warps take part in the ballots
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_up; i += stride) {
        const bool is_if = i < a.N && (a.ntype[i] & HB_TYPE_MASK) == HB_T_INTERFACE;
        list_push(a, list, count, is_if, (uint32_t)i);
    }
}

// K1 on the list: one thread per interface cell, its 18 links in order; the sum runs in
// link order, as updateMass adds its terms, so each cell's new mass is the reference's
// expression.  (One cell per thread rather than one per warp: the FP64 work of a cell
// then shares its warp instructions with 31 other cells on this part's narrow FP64 pipe.)
template <class P>
__global__ void __launch_bounds__(256) k_fs_mass_list(FsArgs a) {
    pdl_enter();
    const int n = cur_count(a);
    const uint32_t* list = cur_list(a);
    const bool first = a.cnt->first != 0;
    for (int w = chunk_first(); w < n; w += chunk_stride()) {
        const Node nd = node_at(a, list[w]);
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
            // av == 0 (either sign) by the bits: an FP64 compare would take the narrow pipe
            if (((unsigned long long)__double_as_longlong(av) << 1) == 0ull) continue;
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
            if (t == HB_T_FLUID) dm += diff;  // av = 1: the product 1.0 * av * diff is diff
            else dm += 1.0 * av * diff;
        }
        a.mass2[i] = mi + dm;
    }
}

// fluid mass = n (LB.cpp:1582-1585): a lean pass over the node bytes, eight per thread
__global__ void __launch_bounds__(256) k_fs_fluid_mass(FsArgs a) {
    pdl_enter();
    const long long nw = (a.N + 7) / 8;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nw; w += (long long)gridDim.x * blockDim.x) {
        const long long i0 = 8 * w;
        uint8_t t[8];
        if (i0 + 8 <= a.N && (a.N & 7) == 0) {
            const uint2 v = reinterpret_cast<const uint2*>(a.ntype)[w];
#pragma unroll
            for (int k = 0; k < 4; ++k) { t[k] = (uint8_t)(v.x >> (8 * k)); t[4 + k] = (uint8_t)(v.y >> (8 * k)); }
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) t[k] = i0 + k < a.N ? a.ntype[i0 + k] : (uint8_t)HB_T_GAS;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if ((t[k] & HB_TYPE_MASK) == HB_T_FLUID) a.mass[i0 + k] = a.rho[i0 + k];
    }
}

// K2 findInterfaceMutants (LB.cpp:1620-1650) over the interface list
__global__ void __launch_bounds__(256) k_fs_classify(FsArgs a) {
    pdl_enter();
    const int n = cur_count(a);
    const uint32_t* list = cur_list(a);
    const int n_up = (n + 31) / 32 * 32;
    for (int w = chunk_first(); w < n_up; w += chunk_stride()) {
        bool conv = false;
        uint32_t iu = 0u;
        if (w < n) {
            iu = list[w];
            const long long i = iu;
            const uint8_t t = a.ntype[i];
            const double m = a.mass2[i];
            a.mass[i] = m;
            if (m > a.rho[i]) {
                a.flag[i] = FS_FILLED;
                a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_FLUID;
                conv = true;
            } else if (m < 0.0) {
                a.flag[i] = FS_EMPTIED;
                a.ntype[i] = (t & ~HB_TYPE_MASK) | HB_T_GAS;
                atomicAdd(&a.cnt->changed, 1);
                conv = true;
            }
        }
        list_push(a, a.clist, &a.cnt->ccount, conv, iu);
    }
}

// K3 smoothenInterface, gas neighbours of filled cells (LB.cpp:1657-1677).  First every
// filled cell m offers itself to its interior gas neighbours g (those whose link back
// along the same direction reaches m: the reference's neighbour table), keeping the
// largest m + 1 per g; then the winner initialises g.
__global__ void __launch_bounds__(256) k_fs_filled_parent(FsArgs a) {
    pdl_enter();
    const int n = min(a.cnt->ccount, (int)a.icap);
    for (int w = chunk_first(); w < n; w += chunk_stride()) {
        const uint32_t m = a.clist[w];
        if (!(a.flag[m] & FS_FILLED)) continue;
        const Node nd = node_at(a, m);
        if (!interior3(a, nd.x, nd.y, nd.z)) continue;
        for (int j = 1; j < Q; ++j) {
            int xg, yg, zg;
            fs_link3(a, nd.x, nd.y, nd.z, j, xg, yg, zg);
            if (!interior3(a, xg, yg, zg)) continue;
            const long long g = lin(a, xg, yg, zg);
            if (code_of(a, g) == HB_T_GAS) atomicMax(a.parent + g, m + 1u);
        }
    }
}

template <class P>
__global__ void __launch_bounds__(256) k_fs_new_from_filled(FsArgs a) {
    pdl_enter();
    const int n = min(a.cnt->ccount, (int)a.icap);
    const int n_up = (n + 31) / 32 * 32;
    for (int w = chunk_first(); w < n_up; w += chunk_stride()) {
        const uint32_t m = w < n ? a.clist[w] : 0u;
        const bool filled = w < n && (a.flag[m] & FS_FILLED);
        const Node nd = node_at(a, m);
        const bool src = filled && interior3(a, nd.x, nd.y, nd.z);
        for (int j = 1; j < Q; ++j) {
            bool mine = false;
            long long g = 0;
            if (src) {
                int xg, yg, zg;
                fs_link3(a, nd.x, nd.y, nd.z, j, xg, yg, zg);
                g = lin(a, xg, yg, zg);
                mine = interior3(a, xg, yg, zg) && a.parent[g] == m + 1u;
            }
            if (mine) {
                const long long i = g, p = m;
                const double F[3] = {a.hf[p] + a.force[0], a.hf[a.N + p] + a.force[1], a.hf[2 * a.N + p] + a.force[2]};
                const double ux = 1.0 * F[0] / 2.0 / 1.0 + a.u[p];  // node::initialize, node.cpp:26-38
                const double uy = 1.0 * F[1] / 2.0 / 1.0 + a.u[a.N + p];
                const double uz = 1.0 * F[2] / 2.0 / 1.0 + a.u[2 * a.N + p];
                const double usq = ux * ux + uy * uy + uz * uz;
                using S = typename P::S;
                S* f = reinterpret_cast<S*>(a.f);
                for (int q = 0; q < Q; ++q) {
                    const double vu = ux * cx(q) + uy * cy(q) + uz * cz(q);
                    double fe = wgt(q) * 1.0 * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
                    if (P::DEV) fe -= wgt(q);
                    P::store(f + (long long)q * a.N + i, (typename P::T)fe);
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
                a.parent[i] = 0u;
                atomicAdd(&a.cnt->changed, 1);
                ledger_add(a, -0.01 * 1.0);
            }
            list_push(a, a.nlist, &a.cnt->ncount, mine, (uint32_t)g);
        }
    }
}

// K4 smoothenInterface, fluid neighbours of emptied cells (LB.cpp:1679-1700); the first
// emptied neighbour to claim a cell (parent slot) converts it
__global__ void __launch_bounds__(256) k_fs_new_from_emptied(FsArgs a) {
    pdl_enter();
    const int n = min(a.cnt->ccount, (int)a.icap);
    const int n_up = (n + 31) / 32 * 32;
    for (int w = chunk_first(); w < n_up; w += chunk_stride()) {
        const uint32_t m = w < n ? a.clist[w] : 0u;
        const bool emptied = w < n && (a.flag[m] & FS_EMPTIED);
        const Node nd = node_at(a, m);
        const bool src = emptied && interior3(a, nd.x, nd.y, nd.z);
        for (int j = 1; j < Q; ++j) {
            bool mine = false;
            long long g = 0;
            if (src) {
                int xg, yg, zg;
                fs_link3(a, nd.x, nd.y, nd.z, j, xg, yg, zg);
                g = lin(a, xg, yg, zg);
                mine = interior3(a, xg, yg, zg) && code_of(a, g) == HB_T_FLUID &&
                       atomicCAS(a.parent + g, 0u, 0xFFFFFFFFu) == 0u;
            }
            if (mine) {
                const double nn = a.rho[g];
                a.mass[g] = 0.99 * nn;
                ledger_add(a, 0.01 * nn);
                a.ntype[g] = (a.ntype[g] & ~HB_TYPE_MASK) | HB_T_INTERFACE;
                a.flag[g] |= FS_NEW_B;
            }
            list_push(a, a.nlist, &a.cnt->ncount, mine, (uint32_t)g);
        }
    }
}

// the interface cells after K3/K4: the step's list minus the converted cells (flag set),
// then the new cells; k indexes that concatenation
__device__ __forceinline__ bool interface_cell(const FsArgs& a, int k, int n0, uint32_t& iu) {
    if (k < n0) {
        iu = cur_list(a)[k];
        return a.flag[iu] == 0;
    }
    iu = a.nlist[k - n0];
    return true;
}

// K5 updateMutants (LB.cpp:1703-1742) over the conversion list, and removeIsolated, first
// pass (LB.cpp:1749-1769) over the interface cells
__global__ void __launch_bounds__(256) k_fs_mutants_to_fluid(FsArgs a) {
    pdl_enter();
    const int nc = min(a.cnt->ccount, (int)a.icap);
    const int n0 = cur_count(a), nn = min(a.cnt->ncount, (int)a.icap);
    const int total = nc + n0 + nn;
    for (int w = chunk_first(); w < total; w += chunk_stride()) {
        if (w < nc) {
            const uint32_t i = a.clist[w];
            const uint8_t fl = a.flag[i];
            if ((fl & FS_EMPTIED) && !(fl & FS_NEW_A)) {
                ledger_add(a, a.mass[i]);
            } else if ((fl & FS_FILLED) && !(fl & FS_NEW_B)) {
                ledger_add(a, a.mass[i] - a.rho[i]);
                a.mass[i] = a.rho[i];
            }
            continue;
        }
        uint32_t iu;
        if (!interface_cell(a, w - nc, n0, iu)) continue;
        const Node nd = node_at(a, iu);
        // all 18 neighbour bytes at once (no early exit: the loads overlap); concurrent
        // conversions in this pass turn interface cells into fluid, never into gas
        bool gas = false;
#pragma unroll
        for (int j = 1; j < Q; ++j) gas |= code_of(a, fs_link(a, nd, j)) == HB_T_GAS;
        if (!gas) {
            ledger_add(a, a.mass[iu] - a.rho[iu]);
            a.mass[iu] = a.rho[iu];
            a.ntype[iu] = (a.ntype[iu] & ~HB_TYPE_MASK) | HB_T_FLUID;
        }
    }
}

// K6 removeIsolated, second pass (LB.cpp:1771-1793); the cells that stay interface form
// the next interface list
__global__ void __launch_bounds__(256) k_fs_isolated_gas(FsArgs a) {
    pdl_enter();
    const int n0 = cur_count(a), nn = min(a.cnt->ncount, (int)a.icap);
    const int total = n0 + nn;
    const int t_up = (total + 31) / 32 * 32;
    uint32_t* next = next_list(a);
    int* ncount = &a.cnt->icount[a.cnt->sel ^ 1];
    for (int w = chunk_first(); w < t_up; w += chunk_stride()) {
        uint32_t iu = 0u;
        bool keep = false;
        if (w < total && interface_cell(a, w, n0, iu) && (a.ntype[iu] & HB_TYPE_MASK) == HB_T_INTERFACE) {
            const Node nd = node_at(a, iu);
            // all 18 neighbour bytes at once (no early exit: the loads overlap); concurrent
            // conversions in this pass turn interface cells into gas, never into fluid
            bool fluid = false;
#pragma unroll
            for (int j = 1; j < Q; ++j) fluid |= code_of(a, fs_link(a, nd, j)) == HB_T_FLUID;
            if (!fluid) {
                ledger_add(a, a.mass[iu]);
                a.ntype[iu] = (a.ntype[iu] & ~HB_TYPE_MASK) | HB_T_GAS;
                atomicAdd(&a.cnt->changed, 1);
            } else {
                keep = true;
            }
        }
        list_push(a, next, ncount, keep, iu);
    }
}

// the surplus and the interface count of the step; the next list becomes current
__global__ void k_fs_ledger(FsArgs a) {
    pdl_enter();
    FsCount* c = a.cnt;
    const int nxt = c->sel ^ 1;
    const long long count = min((long long)c->icount[nxt], a.icap);
    unsigned long long lo = c->ledger[0], hi = c->ledger[1];
    const bool neg = (long long)hi < 0;
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    double surplus = ((double)hi * 18446744073709551616.0 + (double)lo) / LEDGER_ONE;
    if (neg) surplus = -surplus;
    a.scal[0] = surplus;
    a.scal[1] = (double)count;
    a.scal[2] = surplus / (double)count;  // redistributeMass adds surplus / count to each cell
    c->first = 0;
    c->valid = 1;
    c->icount[c->sel] = 0;  // the retired list is the next step's "next"
    c->sel = nxt;
}

// K7 redistributeMass (LB.cpp:1796-1804): the quotient surplus / count is formed once
// (k_fs_ledger), as the reference forms addMass once; then the step's conversion flags
// and claim slots go back to zero
__global__ void __launch_bounds__(256) k_fs_redistribute(FsArgs a) {
    pdl_enter();
    const int n0 = cur_count(a);
    const int nc = min(a.cnt->ccount, (int)a.icap), nn = min(a.cnt->ncount, (int)a.icap);
    const uint32_t* list = cur_list(a);
    const double add = a.scal[2];
    for (int w = chunk_first(); w < n0 + nc + nn; w += chunk_stride()) {
        if (w < n0) {
            a.mass[list[w]] += add;
        } else if (w < n0 + nc) {
            a.flag[a.clist[w - n0]] = 0;
        } else {
            const uint32_t g = a.nlist[w - n0 - nc];
            a.flag[g] = 0;
            a.parent[g] = 0u;
        }
    }
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
    a.scal = c->fs_scal;
    a.force = c->fs_force;
    a.cnt = reinterpret_cast<FsCount*>(c->fs_first);
    a.ilist = c->fs_ilist;
    a.clist = c->fs_ilist + 2 * c->fs_icap;
    a.nlist = c->fs_ilist + 3 * c->fs_icap;
    a.parent = c->fs_parent;
    a.icap = c->fs_icap;
    a.status = c->status;
    return a;
}

size_t fs_count_bytes() { return 64; }

// the interface list is rebuilt from the node bytes at the next step (after an upload of
// the node types or a restore)
void fs_invalidate(hb_ctx* c) {
    if (!c->fs_first) return;
    FsCount h = {};
    cudaMemcpy(&h, c->fs_first, sizeof(h), cudaMemcpyDeviceToHost);
    h.valid = 0;
    h.icount[0] = h.icount[1] = 0;
    cudaMemcpy(c->fs_first, &h, sizeof(h), cudaMemcpyHostToDevice);
}

// a checkpoint carries no interface list (the loader rebuilds it from the node bytes),
// so its copy of the step state says so, whichever list was current
void fs_count_for_file(void* rec) {
    FsCount* h = static_cast<FsCount*>(rec);
    h->valid = 0;
    h->sel = 0;
    h->icount[0] = h->icount[1] = 0;
}

int fs_init(hb_ctx* c) {
    const long long N = c->N;
    c->fs_icap = c->P.cap_interface > 0 ? std::min<long long>(c->P.cap_interface, N) : N;
    if (cudaMalloc(&c->fs_flag, N) != cudaSuccess || cudaMalloc(&c->fs_mass2, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&c->fs_scal, sizeof(double) * 3) != cudaSuccess ||
        cudaMalloc(&c->fs_first, fs_count_bytes()) != cudaSuccess ||
        cudaMalloc(&c->fs_parent, sizeof(uint32_t) * N) != cudaSuccess ||
        cudaMalloc(&c->fs_ilist, sizeof(uint32_t) * 4 * c->fs_icap) != cudaSuccess)
        return HB_ERR_NOMEM;
    cudaMemset(c->fs_flag, 0, N);
    cudaMemset(c->fs_parent, 0, sizeof(uint32_t) * N);
    cudaMemset(c->fs_scal, 0, sizeof(double) * 3);
    FsCount h = {};
    h.first = 1;  // first step; the interface list is built at the first step
    cudaMemset(c->fs_first, 0, fs_count_bytes());
    cudaMemcpy(c->fs_first, &h, sizeof(h), cudaMemcpyHostToDevice);
    return cudaGetLastError() == cudaSuccess ? HB_OK : HB_ERR_CUDA;
}

void launch_fs_step(hb_ctx* c, int cur) {
    FsArgs a = fs_args(c, cur);
    cudaStream_t s = c->stream;
    const int GL = FS_LIST_GRID;
    // this step's conversion and new-cell counts and its ledger start at zero
    cudaMemsetAsync(&a.cnt->ccount, 0, sizeof(FsCount) - offsetof(FsCount, ccount), s);
    // a chain of short list passes: each one scheduled behind the tail of the previous
    launch_pdl(k_fs_ilist, GL, 256, s, a);
    if (c->P.precision == HB_FP64) launch_pdl(k_fs_mass_list<PolF64>, GL, 256, s, a);
    else if (c->P.precision == HB_FP32) launch_pdl(k_fs_mass_list<PolF32>, GL, 256, s, a);
    else launch_pdl(k_fs_mass_list<PolF16>, GL, 256, s, a);
    launch_pdl(k_fs_fluid_mass, 152 * 8, 256, s, a);
    launch_pdl(k_fs_classify, GL, 256, s, a);
    launch_pdl(k_fs_filled_parent, GL, 256, s, a);
    if (c->P.precision == HB_FP64) launch_pdl(k_fs_new_from_filled<PolF64>, GL, 256, s, a);
    else if (c->P.precision == HB_FP32) launch_pdl(k_fs_new_from_filled<PolF32>, GL, 256, s, a);
    else launch_pdl(k_fs_new_from_filled<PolF16>, GL, 256, s, a);
    launch_pdl(k_fs_new_from_emptied, GL, 256, s, a);
    launch_pdl(k_fs_mutants_to_fluid, GL, 256, s, a);
    launch_pdl(k_fs_isolated_gas, GL, 256, s, a);
    launch_pdl(k_fs_ledger, 1, 1, s, a);
    launch_pdl(k_fs_redistribute, GL, 256, s, a);
    launch_refresh_bulk(c, &a.cnt->changed);  // only when a cell's activity changed
}

}  // namespace hb
