// hb_slip.cu -- slip walls, boundary codes 5 (static) and 6 (moving; LB.cpp:1358-1456).
//
// In the reference a population fs[j] that leaves node i toward a slip wall comes back
// as f[opp j] = fs[j] (bounce-back), except on a diagonal link with exactly one of its two
// axis neighbours c active: then f[opp j] = S1 fs_c[d] + S2 fs[j], where d is j with the
// component along c reversed -- the population of c that is reflected off the wall into
// i (specular part S1 = slipCoefficient, S2 = 1 - S1).  Moving slip walls subtract BBi
// from fs[j]; the walls built from boundary codes have zero velocity (DEM.cpp:452-457), so
// BBi is zero and both codes stream alike.
//
// The lattice kernels push: node i's kernel thread cannot read c's post-collision
// values.  So the lattice kernels bounce every slip link back unchanged (f_out[opp j][i]
// = fs[j], exactly as a static wall), and after them one pass over the static list of
// (node, diagonal slip link) entries mixes the two bounced-back values: c's own slip link
// in direction d ends on the same wall, so its bounce-back slot f_out[opp d][c] holds
// fs_c[d].  The pass reads every input first (pass A into a side array) and writes after
// (pass B), because pairs of entries read each other's slots.
#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

__host__ __device__ constexpr int dir_of(int x, int y, int z) {
    int r = -1;
    for (int j = 0; j < Q; ++j)
        if (cx(j) == x && cy(j) == y && cz(j) == z) r = j;
    return r;
}

// along the k-th non-zero axis of diagonal j: the axis neighbour to check and the partner
// direction (j with that component reversed); the reference's lattice.h:87-94 tables
__host__ __device__ constexpr void slip_pair(int j, int k, int& check, int& dir) {
    const int c[3] = {cx(j), cy(j), cz(j)};
    int n = 0;
    check = dir = 0;
    for (int a = 0; a < 3; ++a) {
        if (!c[a]) continue;
        if (n == k) {
            int u[3] = {0, 0, 0}, f[3] = {c[0], c[1], c[2]};
            u[a] = c[a];
            f[a] = -c[a];
            check = dir_of(u[0], u[1], u[2]);
            dir = dir_of(f[0], f[1], f[2]);
        }
        ++n;
    }
}

__device__ __forceinline__ bool slip_code(uint8_t c) { return c == HB_T_SLIPSTAT || c == HB_T_SLIPDYN; }

struct SlipArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    const uint8_t* ntype;
    void* f;                        // populations after the lattice step
    const unsigned long long* list; // node * 32 + j
    int count;
    double* val;                    // mixed values (pass A -> pass B)
    uint8_t* mix;                   // 1: entry mixes this step
    double S1, S2;
    int* status;
};

__device__ __forceinline__ long long slip_link(const SlipArgs& a, long long i, int j) {
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
    if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
    if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
    if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
    return (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
}

// entries: interior non-wall nodes (any of them can be active now or later) and their
// diagonal links that end on a slip wall; walls never change, so the list is built once
__global__ void k_slip_list(SlipArgs a, unsigned long long* list, int* count, int cap) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    if (x < 1 || y < 1 || z < 1 || x > a.X - 2 || y > a.Y - 2 || z > a.Z - 2) return;
    const uint8_t t = a.ntype[i] & HB_TYPE_MASK;
    if (t >= 5 && t <= 9) return;
    for (int j = 7; j < Q; ++j) {
        if (!slip_code(a.ntype[slip_link(a, i, j)] & HB_TYPE_MASK)) continue;
        const int k = atomicAdd(count, 1);
        if (k < cap) list[k] = (unsigned long long)i * 32ull + (unsigned long long)j;
    }
}

template <class P>
__global__ void k_slip_mix(SlipArgs a) {
    using S = typename P::S;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.count) return;
    const long long i = (long long)(a.list[k] >> 5);
    const int j = (int)(a.list[k] & 31ull);
    uint8_t m = 0;
    if (is_active(a.ntype[i])) {
        int ch0, d0, ch1, d1;
        slip_pair(j, 0, ch0, d0);
        slip_pair(j, 1, ch1, d1);
        const long long c0 = slip_link(a, i, ch0), c1 = slip_link(a, i, ch1);
        const bool a0 = is_active(a.ntype[c0]), a1 = is_active(a.ntype[c1]);
        if (a0 != a1) {
            const long long c = a0 ? c0 : c1;
            const int d = a0 ? d0 : d1;
            // the partner's own link d must end on a wall that bounced fs_c[d] back as is
            // (static, slip or curved: the curved pass runs after this one)
            const uint8_t pl = a.ntype[slip_link(a, c, d)] & HB_TYPE_MASK;
            if (!(slip_code(pl) || pl == HB_T_STATWALL || pl == HB_T_CURVED)) flag_status(a.status, 1);
            const S* f = reinterpret_cast<const S*>(a.f);
            const double fp = (double)P::load(f + (long long)opp(d) * a.N + c);
            const double fo = (double)P::load(f + (long long)opp(j) * a.N + i);
            // FP32/FP16: deviations from w; both directions are diagonals (same w) and
            // S1 + S2 = 1, so the mixture of deviations is the deviation of the mixture
            a.val[k] = a.S1 * fp + a.S2 * fo;
            m = 1;
        }
    }
    a.mix[k] = m;
}

template <class P>
__global__ void k_slip_store(SlipArgs a) {
    using S = typename P::S;
    using T = typename P::T;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.count || !a.mix[k]) return;
    const long long i = (long long)(a.list[k] >> 5);
    const int j = (int)(a.list[k] & 31ull);
    P::store(reinterpret_cast<S*>(a.f) + (long long)opp(j) * a.N + i, (T)a.val[k]);
}

static SlipArgs slip_args(hb_ctx* c, void* f) {
    SlipArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype;
    a.f = f;
    a.list = c->slip_list;
    a.count = c->slip_n;
    a.val = c->slip_val;
    a.mix = c->slip_mix;
    a.S1 = c->P.slip_coefficient;
    a.S2 = 1.0 - c->P.slip_coefficient;  // LB.cpp:1154-1155
    a.status = c->status;
    return a;
}

int slip_init(hb_ctx* c) {
    bool any = false;
    for (int k = 0; k < 6; ++k) any |= c->P.boundary[k] == HB_T_SLIPSTAT || c->P.boundary[k] == HB_T_SLIPDYN;
    c->slip_n = 0;
    if (!any) return 0;
    int* cnt = nullptr;
    if (cudaMalloc(&cnt, sizeof(int)) != cudaSuccess) return -1;
    cudaMemset(cnt, 0, sizeof(int));
    SlipArgs a = slip_args(c, nullptr);
    const unsigned G = (unsigned)ceil_div(c->N, 256);
    k_slip_list<<<G, 256, 0, c->stream>>>(a, nullptr, cnt, 0);
    int n = 0;
    cudaMemcpyAsync(&n, cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    if (n > 0) {
        if (cudaMalloc(&c->slip_list, sizeof(unsigned long long) * n) != cudaSuccess ||
            cudaMalloc(&c->slip_val, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&c->slip_mix, (size_t)n) != cudaSuccess) {
            cudaFree(cnt);
            return -1;
        }
        cudaMemsetAsync(cnt, 0, sizeof(int), c->stream);
        k_slip_list<<<G, 256, 0, c->stream>>>(a, c->slip_list, cnt, n);
        cudaStreamSynchronize(c->stream);
    }
    cudaFree(cnt);
    c->slip_n = n;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void launch_slip(hb_ctx* c, void* f) {
    if (c->slip_n == 0) return;
    const SlipArgs a = slip_args(c, f);
    const unsigned G = (unsigned)ceil_div(c->slip_n, 128);
    if (c->P.precision == HB_FP64) {
        k_slip_mix<PolF64><<<G, 128, 0, c->stream>>>(a);
        k_slip_store<PolF64><<<G, 128, 0, c->stream>>>(a);
    } else if (c->P.precision == HB_FP32) {
        k_slip_mix<PolF32><<<G, 128, 0, c->stream>>>(a);
        k_slip_store<PolF32><<<G, 128, 0, c->stream>>>(a);
    } else {
        k_slip_mix<PolF16><<<G, 128, 0, c->stream>>>(a);
        k_slip_store<PolF16><<<G, 128, 0, c->stream>>>(a);
    }
}

}  // namespace hb
