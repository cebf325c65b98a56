// hb_io.cu -- output mirror: what the reference's IO reads from the solver at an output
// step, computed and packed on the device so that an output step costs one kernel pass
// and one copy instead of a host walk over every node object.
//   fluid image data (IO::exportParaviewFluidOld, IO.cpp:698-831): type, v, pressure,
//     dynVisc, mass, solidIndex per lattice node;
//   export.dat quantities (IO::outputStep, IO.cpp:132-198, 835-1104): fluid and particle
//     maximum speeds, total fluid mass, plastic fraction, collision / hydraulic force
//     totals, particle mass, obstacle force, and the particle energies of
//     DEM::updateEnergy (DEM.cpp:2226-2276).
// FP64 expressions keep the reference's evaluation order (this file is compiled without
// FMA contraction).  Element sums run on one thread in element order, the reference's
// own order; node sums use fixed per-thread ranges, a fixed block tree and a fixed
// block order.
#include <cstdio>
#include <fstream>
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {

// nodeType::isWall (node.cpp:318-320): slip/static/moving/curved walls
__device__ __forceinline__ bool is_wall_code(uint8_t c) { return c >= 5 && c <= 9; }

struct IoArgs {
    int X, Y, Z;
    long long N;
    int per[6];
    const uint8_t* ntype;
    const uint32_t* solid;
    const double* rho;
    const double* u;
    const double* mass;
    const void* visc;
    int visc_kind;      // 0: no viscosity field (constant initial value), 1: float, 2: double
    double init_visc;
    uint8_t* linked;    // [N] 1: a wall node that a non-wall node links to
};

// LB::initializeWalls (LB.cpp:946-995): a wall node owns a node object (and so prints its
// own values) when a non-wall node links to it.  Links as LB::initializeLatticeBoundaries:
// interior nodes link arithmetically with the periodic remap, boundary nodes to
// themselves.  Walls never change type, so the marks are computed once.
__global__ void k_io_linked(IoArgs a) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const int x = (int)(i % a.X), y = (int)((i / a.X) % a.Y), z = (int)(i / ((long long)a.X * a.Y));
    if (x < 1 || y < 1 || z < 1 || x > a.X - 2 || y > a.Y - 2 || z > a.Z - 2) return;
    if (is_wall_code(a.ntype[i] & HB_TYPE_MASK)) return;
    for (int j = 1; j < Q; ++j) {
        int xn = x + cx(j), yn = y + cy(j), zn = z + cz(j);
        if (xn == 0 && a.per[0]) xn = a.X - 2; else if (xn == a.X - 1 && a.per[1]) xn = 1;
        if (yn == 0 && a.per[2]) yn = a.Y - 2; else if (yn == a.Y - 1 && a.per[3]) yn = 1;
        if (zn == 0 && a.per[4]) zn = a.Z - 2; else if (zn == a.Z - 1 && a.per[5]) zn = 1;
        const long long l = (long long)xn + (long long)a.X * ((long long)yn + (long long)a.Y * zn);
        if (is_wall_code(a.ntype[l] & HB_TYPE_MASK)) a.linked[l] = 1;
    }
}

__device__ __forceinline__ double node_visc(const IoArgs& a, long long i) {
    if (a.visc_kind == 1) return (double)reinterpret_cast<const float*>(a.visc)[i];
    if (a.visc_kind == 2) return reinterpret_cast<const double*>(a.visc)[i];
    return a.init_visc;
}

// 0: no node object, 1: fluid/interface node, 2: wall node with an object
__device__ __forceinline__ int node_kind(const IoArgs& a, long long i, uint8_t code) {
    if (code == HB_T_FLUID || code == HB_T_INTERFACE) return 1;
    if (is_wall_code(code) && a.linked[i]) return 2;
    return 0;
}

struct VtkOut {
    int8_t* type;       // [N]
    double* v;          // [3N] x, y, z per node (the order the file lists them)
    double* pressure;   // [N]
    double* visc;       // [N]
    double* mass;       // [N]
    uint32_t* solid;    // [N]
};

// IO.cpp:721-819 per node: type (1 inside a particle), velocity, 0.3333333 (n - 1),
// viscosity and mass of the node object, zero where there is none.  Wall objects are
// initialised with density 1, zero mass and viscosity and the wall velocity
// (LB.cpp:958-990); in lattice units every unit factor is 1.
__global__ void k_io_pack(IoArgs a, VtkOut o) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const uint8_t t = a.ntype[i];
    const uint8_t code = t & HB_TYPE_MASK;
    const int kind = node_kind(a, i, code);
    double vx = 0.0, vy = 0.0, vz = 0.0, p = 0.0, vi = 0.0, m = 0.0;
    if (kind == 1) {
        vx = a.u[i]; vy = a.u[a.N + i]; vz = a.u[2 * a.N + i];
        const double n = a.rho[i];
        p = n != 0.0 ? 0.3333333 * (n - 1.0) * 1.0 : n;
        vi = node_visc(a, i);
        m = a.mass[i];
    } else if (kind == 2) {
        if (code == HB_T_DYNWALL) { vx = a.u[i]; vy = a.u[a.N + i]; vz = a.u[2 * a.N + i]; }
        p = 0.3333333 * (1.0 - 1.0) * 1.0;
    }
    if (o.type) o.type[i] = (t & HB_INSIDE) ? (int8_t)1 : (int8_t)code;
    if (o.v) { o.v[3 * i] = vx; o.v[3 * i + 1] = vy; o.v[3 * i + 2] = vz; }
    if (o.pressure) o.pressure[i] = p;
    if (o.visc) o.visc[i] = vi;
    if (o.mass) o.mass[i] = m;
    if (o.solid) o.solid[i] = a.solid[i];
}

// ---- export.dat quantities -------------------------------------------------------------

constexpr int IO_BLOCKS = 456;  // 3 x 152 SMs
constexpr int IO_THREADS = 256;

struct NodePart {
    double maxu2, mass;
    long long active, plastic;
};

// Per block: max |u|^2 over active nodes (IO.cpp:835-851), the fluid mass of active nodes
// outside particles (IO.cpp:987-999), the active count and the nodes above 0.95 of the
// maximum viscosity (IO.cpp:969-985).  Each thread takes a fixed contiguous range of
// nodes, so the sums do not depend on scheduling.
__global__ void __launch_bounds__(IO_THREADS) k_io_nodes(IoArgs a, double visc_cut, NodePart* part) {
    __shared__ double s_max[IO_THREADS], s_mass[IO_THREADS];
    __shared__ long long s_act[IO_THREADS], s_pl[IO_THREADS];
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (a.N + T - 1) / T;
    const long long i0 = t * per, i1 = min(a.N, i0 + per);
    double mx = 0.0, ms = 0.0;
    long long act = 0, pl = 0;
    for (long long i = i0; i < i1; ++i) {
        const uint8_t tt = a.ntype[i];
        const uint8_t code = tt & HB_TYPE_MASK;
        if (code != HB_T_FLUID && code != HB_T_INTERFACE) continue;
        const double ux = a.u[i], uy = a.u[a.N + i], uz = a.u[2 * a.N + i];
        mx = fmax(mx, ux * ux + uy * uy + uz * uz);
        if (!(tt & HB_INSIDE)) ms += a.mass[i];
        ++act;
        if (node_visc(a, i) > visc_cut) ++pl;
    }
    s_max[threadIdx.x] = mx; s_mass[threadIdx.x] = ms; s_act[threadIdx.x] = act; s_pl[threadIdx.x] = pl;
    __syncthreads();
    for (int q = IO_THREADS / 2; q > 0; q >>= 1) {
        if ((int)threadIdx.x < q) {
            s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + q]);
            s_mass[threadIdx.x] += s_mass[threadIdx.x + q];
            s_act[threadIdx.x] += s_act[threadIdx.x + q];
            s_pl[threadIdx.x] += s_pl[threadIdx.x + q];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = NodePart{s_max[0], s_mass[0], s_act[0], s_pl[0]};
}

struct IoElem {
    int E, O;
    const double *x0, *x1, *wG, *wL, *I, *m, *FH, *FP, *FW;
    const double* react;  // objects' FParticle at react + 3*MAX_WALLS
    double demF[3];
    double size[3];       // demSize (DEM.cpp:190-192)
};

// Layout of the device result block (doubles); hb_export_values copies it field by field.
enum IoSlot {
    S_MAXU2, S_FMASS, S_ACTIVE, S_PLASTIC, S_PMAX2, S_WMAX2, S_COLL, S_HYDR, S_PMASS,
    S_OBJX, S_OBJY, S_OBJZ, S_TRKIN, S_ROTKIN, S_GRAV, S_COUNT
};

__device__ __forceinline__ double n2(double x, double y, double z) { return x * x + y * y + z * z; }

// Element terms of IO.cpp:853-876, 1001-1010, 1064-1106 and DEM.cpp:2226-2276, one thread
// per element (the sums over elements are formed afterwards in element order):
// [0] |FParticle| [1] |FWall| [2] |FHydro| [3] m [4] 0.5 m |x1|^2 [5] I.(wL*wL) [6] m h |g|
constexpr int IO_TERMS = 7;
__global__ void k_io_terms(IoElem e, double* terms, double* maxima) {
    const int E = e.E;
    const double gn = sqrt(n2(e.demF[0], e.demF[1], e.demF[2]));
    double zn[3] = {0.0, 0.0, 0.0}, zp[3] = {0.0, 0.0, 0.0};
    if (gn != 0.0) {  // reference plane of the gravitational energy (DEM.cpp:2248-2264)
        for (int k = 0; k < 3; ++k) zn[k] = -1.0 * e.demF[k] / gn;
        for (int k = 0; k < 3; ++k)
            if (zn[k] < 0) zp[k] += e.size[k];
    }
    double pmax = 0.0, wmax = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const double vx = e.x1[i], vy = e.x1[E + i], vz = e.x1[2 * E + i];
        pmax = fmax(pmax, n2(vx, vy, vz));
        wmax = fmax(wmax, n2(e.wG[i], e.wG[E + i], e.wG[2 * E + i]));
        double* t = terms + (long long)IO_TERMS * i;
        t[0] = sqrt(n2(e.FP[i], e.FP[E + i], e.FP[2 * E + i]));
        t[1] = sqrt(n2(e.FW[i], e.FW[E + i], e.FW[2 * E + i]));
        t[2] = sqrt(n2(e.FH[i], e.FH[E + i], e.FH[2 * E + i]));
        t[3] = e.m[i];
        t[4] = 0.5 * e.m[i] * n2(vx, vy, vz);
        const double wx = e.wL[i], wy = e.wL[E + i], wz = e.wL[2 * E + i];
        t[5] = e.I[i] * (wx * wx) + e.I[E + i] * (wy * wy) + e.I[2 * E + i] * (wz * wz);
        t[6] = 0.0;
        if (gn != 0.0) {
            const double h = zn[0] * (e.x0[i] - zp[0]) + zn[1] * (e.x0[E + i] - zp[1]) + zn[2] * (e.x0[2 * E + i] - zp[2]);
            t[6] = e.m[i] * h * gn;
        }
    }
    // maxima are order-independent: warp shuffles, then 64-bit atomicMax on the bit patterns
    // of the non-negative values
    for (int off = 16; off > 0; off >>= 1) {
        pmax = fmax(pmax, __shfl_xor_sync(0xffffffffu, pmax, off));
        wmax = fmax(wmax, __shfl_xor_sync(0xffffffffu, wmax, off));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(reinterpret_cast<unsigned long long*>(maxima), (unsigned long long)__double_as_longlong(pmax));
        atomicMax(reinterpret_cast<unsigned long long*>(maxima + 1), (unsigned long long)__double_as_longlong(wmax));
    }
}

// One thread: the block partials in block order, then the element sums in element order
// (the reference's own accumulation order; the terms come from k_io_terms).
__global__ void k_io_final(const NodePart* part, int nparts, IoElem e, const double* terms, const double* maxima,
                           double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double mx = 0.0, ms = 0.0;
    long long act = 0, pl = 0;
    for (int b = 0; b < nparts; ++b) {
        mx = fmax(mx, part[b].maxu2);
        ms += part[b].mass;
        act += part[b].active;
        pl += part[b].plastic;
    }
    out[S_MAXU2] = mx; out[S_FMASS] = ms; out[S_ACTIVE] = (double)act; out[S_PLASTIC] = (double)pl;
    double coll = 0.0, hydr = 0.0, pmass = 0.0, tKin = 0.0, rKin = 0.0, g = 0.0;
    for (int i = 0; i < e.E; ++i) {
        const double* t = terms + (long long)IO_TERMS * i;
        coll += t[0];
        coll += t[1];
        hydr += t[2];
        pmass += t[3];
        tKin += t[4];
        rKin += t[5];
        g += t[6];
    }
    double ox = 0.0, oy = 0.0, oz = 0.0;  // IO::totForceObject (IO.cpp:1097-1106)
    if (e.react)
        for (int o = 0; o < e.O; ++o) {
            const double* f = e.react + 3 * (MAX_WALLS + o);
            ox += f[0]; oy += f[1]; oz += f[2];
        }
    out[S_PMAX2] = e.E ? maxima[0] : 0.0;
    out[S_WMAX2] = e.E ? maxima[1] : 0.0;
    out[S_COLL] = coll; out[S_HYDR] = hydr; out[S_PMASS] = pmass;
    out[S_OBJX] = ox; out[S_OBJY] = oy; out[S_OBJZ] = oz;
    out[S_TRKIN] = tKin; out[S_ROTKIN] = rKin; out[S_GRAV] = g;
}

static IoArgs io_args(hb_ctx* c) {
    IoArgs a;
    a.X = c->X; a.Y = c->Y; a.Z = c->Z; a.N = c->N;
    for (int k = 0; k < 6; ++k) a.per[k] = c->P.boundary[k] == HB_T_PERIODIC;
    a.ntype = c->ntype; a.solid = c->solid; a.rho = c->rho; a.u = c->u; a.mass = c->mass;
    a.visc = c->visc;
    a.visc_kind = c->visc ? (c->P.precision == HB_FP64 ? 2 : 1) : 0;
    a.init_visc = c->P.init_visc;
    a.linked = c->io_linked;
    return a;
}

int io_prepare(hb_ctx* c) {
    if (c->io_part) return 0;
    if (cudaMalloc(&c->io_part, sizeof(NodePart) * IO_BLOCKS + sizeof(double) * (S_COUNT + 2)) != cudaSuccess)
        return -1;
    if (c->d.E > 0 && cudaMalloc(&c->io_terms, sizeof(double) * IO_TERMS * c->d.E) != cudaSuccess) return -1;
    if (!c->P.lb_solve || !c->ntype) return 0;  // DEM only: no lattice nodes
    if (cudaMalloc(&c->io_linked, (size_t)c->N) != cudaSuccess) return -1;
    cudaMemsetAsync(c->io_linked, 0, (size_t)c->N, c->stream);
    const IoArgs a = io_args(c);
    k_io_linked<<<(unsigned)ceil_div(c->N, 256), 256, 0, c->stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void launch_io_pack(hb_ctx* c, int8_t* type, double* v, double* pressure, double* visc, double* mass,
                    uint32_t* solid) {
    const IoArgs a = io_args(c);
    const VtkOut o{type, v, pressure, visc, mass, solid};
    k_io_pack<<<(unsigned)ceil_div(c->N, 256), 256, 0, c->stream>>>(a, o);
}

// the export.dat quantities into out[S_COUNT] (device), queued on the context stream
double* launch_io_export(hb_ctx* c) {
    const IoArgs a = io_args(c);
    NodePart* part = reinterpret_cast<NodePart*>(c->io_part);
    double* out = reinterpret_cast<double*>(part + IO_BLOCKS);
    const double visc_cut = 0.95 * ((1.8 - 0.5) / 3 / 1.0);  // IO.cpp:971, maxTau 1.8 (lattice.h:30)
    if (c->io_linked) k_io_nodes<<<IO_BLOCKS, IO_THREADS, 0, c->stream>>>(a, visc_cut, part);
    else cudaMemsetAsync(part, 0, sizeof(NodePart) * IO_BLOCKS, c->stream);
    IoElem e = {};
    const hb_dem_dev& d = c->d;
    e.E = d.E; e.O = d.O;
    if (d.E > 0) {
        e.x0 = d.x[0]; e.x1 = d.x[1]; e.wG = d.wG; e.wL = d.wL; e.I = d.I; e.m = d.m;
        e.FH = d.FH; e.FP = d.FP; e.FW = d.FW; e.react = d.react;
    }
    for (int k = 0; k < 3; ++k) {
        e.demF[k] = c->P.lbF[k];  // DEM.cpp:194
        e.size[k] = double(c->P.lb_size[k]) * 1.0;
    }
    double* maxima = out + S_COUNT;
    cudaMemsetAsync(maxima, 0, 2 * sizeof(double), c->stream);
    if (d.E > 0) k_io_terms<<<(unsigned)ceil_div(d.E, 256), 256, 0, c->stream>>>(e, c->io_terms, maxima);
    k_io_final<<<1, 32, 0, c->stream>>>(part, IO_BLOCKS, e, c->io_terms, maxima, out);
    return out;
}

int io_slot_count() { return S_COUNT; }

}  // namespace hb
