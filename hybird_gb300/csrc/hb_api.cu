// hb_api.cu -- the C-ABI (include/hybird_gpu.h): context lifecycle, initial state,
// whole-cycle CUDA graph, downloads, status and timing.
//
// One cycle is the reference's goCycle (hybird.cpp:35-66) minus output:
//   DEM substeps -> free-surface step -> coupling masks -> collide+stream -> element
//   (element forces of the previous step, DEM substeps and coupling masks in one
//   cooperative kernel) -> free surface -> collide+stream.
// It is captured once into a CUDA graph and replayed; all device memory is allocated in
// hb_create/hb_init, nothing per step.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <locale>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace {
thread_local std::string g_err;

int seterr(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t _e = (call);                                                      \
        if (_e != cudaSuccess)                                                        \
            return seterr(HB_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                          __FILE__, __LINE__);                                        \
    } while (0)

}  // namespace

namespace hb {
int set_error(int code, const char* msg) { return seterr(code, "%s", msg); }
}  // namespace hb

namespace {

template <class T>
int dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e != cudaSuccess) return seterr(HB_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
    return HB_OK;
}

int check_params(const hb_params* p) {
    for (int k = 0; k < 3; ++k)
        if (p->lb_size[k] < 3) return seterr(HB_ERR_ARG, "lb_size[%d] = %d < 3", k, p->lb_size[k]);
    for (int k = 0; k < 3; ++k)  // node coordinates travel as 16-bit values in the mask queues
        if (p->lb_size[k] > 65535) return seterr(HB_ERR_UNSUPPORTED, "lb_size[%d] = %d > 65535", k, p->lb_size[k]);
    for (int k = 0; k < 3; ++k)
        if (p->units[k] != 1.0) return seterr(HB_ERR_UNSUPPORTED, "units must be 1 (lattice units)");
    for (int k = 0; k < 6; ++k) {
        const int b = p->boundary[k];
        if (b != HB_T_PERIODIC && !(b >= HB_T_SLIPSTAT && b <= HB_T_DYNWALL))
            return seterr(HB_ERR_UNSUPPORTED, "boundary%d = %d: only 4 (periodic), 5, 6 (slip), 7, 8 are implemented",
                          k, b);
    }
    if (!(p->slip_coefficient >= 0.0 && p->slip_coefficient <= 1.0)) return seterr(HB_ERR_ARG, "slip_coefficient");
    for (int k = 0; k < 6; ++k)
        if (p->free_surface && p->boundary[k] == HB_T_SLIPDYN)
            return seterr(HB_ERR_UNSUPPORTED, "moving slip walls (6) with a free surface are not implemented");
    if (!(p->init_visc > 0.0)) return seterr(HB_ERR_ARG, "init_visc must be > 0");
    if (p->precision < HB_FP64 || p->precision > HB_FP16S) return seterr(HB_ERR_ARG, "precision");
    if (p->collision != HB_BGK && p->collision != HB_TRT) return seterr(HB_ERR_ARG, "collision");
    if (p->dem_solve && (p->multi_step < 1 || p->multi_step > hb::MAX_MULTI))
        return seterr(HB_ERR_ARG, "multi_step must be in 1..%d", hb::MAX_MULTI);
    if (p->cap_neighbors < 0 || p->cap_neighbors > 4096) return seterr(HB_ERR_ARG, "cap_neighbors must be in 0..4096");
    if (p->coupling != HB_DIRECT_FORCING && p->coupling != HB_MOVING_BB) return seterr(HB_ERR_ARG, "coupling");
    if (p->coupling == HB_MOVING_BB && p->free_surface)
        return seterr(HB_ERR_UNSUPPORTED, "moving bounce-back coupling with a free surface is not implemented");
    if (p->cap_interface < 0) return seterr(HB_ERR_ARG, "cap_interface must be >= 0");
    const long long N = (long long)p->lb_size[0] * p->lb_size[1] * p->lb_size[2];
    if (p->precision != HB_FP64 && 19LL * N >= (1LL << 31))  // 32-bit population offsets
        return seterr(HB_ERR_UNSUPPORTED, "FP32/FP16 lattices are limited to 19 * nodes < 2^31 (%lld nodes)", N);
    return HB_OK;
}
}  // namespace

namespace hb {

int dem_init(hb_ctx* c, const hb_elements* e, const hb_objects* o) {
    hb_dem_dev& d = c->d;
    const hb_params& P = c->P;
    // walls from the boundary codes (DEM.cpp:435-633)
    const double ps[6][3] = {{0.5, 0, 0}, {c->X - 1.5, 0, 0}, {0, 0.5, 0}, {0, c->Y - 1.5, 0}, {0, 0, 0.5}, {0, 0, c->Z - 1.5}};
    const double ns[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    d.nw = 0;
    for (int k = 0; k < 6; ++k) {
        const int b = P.boundary[k];
        if (b == HB_T_SLIPSTAT || b == HB_T_SLIPDYN || b == HB_T_STATWALL || b == HB_T_DYNWALL) {
            for (int q = 0; q < 3; ++q) { d.wall_p[d.nw][q] = ps[k][q]; d.wall_n[d.nw][q] = ns[k][q]; }
            d.wall_code[d.nw] = b;
            ++d.nw;
        }
    }
    const double re = P.restitution;
    d.dampCoeff = -1.0 * std::sqrt(2.0) * std::log(re) / std::sqrt((std::log(re) * std::log(re) + M_PI));
    d.knConst = 2.0 / 3.0 * P.young_mod / (1 - P.poisson * P.poisson);
    d.ksConst = 2.0 * P.young_mod / (2.0 - P.poisson) / (1.0 + P.poisson);
    // objects (host copies: periodic images are appended once nebrRange is known)
    const int O0 = o ? o->count : 0;
    std::vector<double> ox(3 * (size_t)O0), ov(3 * (size_t)O0, 0.0), orr(O0);
    for (int k = 0; k < O0; ++k) {
        for (int q = 0; q < 3; ++q) {
            ox[3 * k + q] = o->x0[(size_t)q * O0 + k];
            if (o->x1) ov[3 * k + q] = o->x1[(size_t)q * O0 + k];
        }
        orr[k] = o->radius[k];
    }
    d.O_std = O0;
    auto upload_objects = [&]() -> int {
        d.O = (int)orr.size();
        if (d.O == 0) return HB_OK;
        int rc;
        if ((rc = dalloc(&d.obj_x0, 3 * d.O)) || (rc = dalloc(&d.obj_x1, 3 * d.O)) || (rc = dalloc(&d.obj_r, d.O))) return rc;
        std::vector<double> a(3 * (size_t)d.O), v(3 * (size_t)d.O);
        for (int k = 0; k < d.O; ++k)
            for (int q = 0; q < 3; ++q) {
                a[(size_t)q * d.O + k] = ox[3 * k + q];
                v[(size_t)q * d.O + k] = ov[3 * k + q];
            }
        CK(cudaMemcpy(d.obj_x0, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.obj_x1, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.obj_r, orr.data(), sizeof(double) * d.O, cudaMemcpyHostToDevice));
        return HB_OK;
    };
    const int E = (P.dem_solve && e) ? e->count : 0;
    d.E = E;
    d.nbr_cap = P.cap_neighbors > 0 ? (int)P.cap_neighbors : NBR_CAP;
    d.multi = E ? P.multi_step : 1;
    d.dt = E ? 1.0 / double(P.multi_step) : 1.0;
    if (E == 0) return upload_objects();
    // periodic face pairs (DEM::initializePbcs, DEM.cpp:937-989), lattice units
    d.npbc = 0;
    {
        const int L[3] = {c->X, c->Y, c->Z};
        for (int k = 0; k < 3; ++k) {
            const bool lo = P.boundary[2 * k] == HB_T_PERIODIC, hi = P.boundary[2 * k + 1] == HB_T_PERIODIC;
            if (lo != hi) return seterr(HB_ERR_UNSUPPORTED, "periodic boundary on one face of axis %d only", k);
            if (!lo) continue;
            for (int q = 0; q < 3; ++q) {
                d.pbc_p[d.npbc][q] = q == k ? 0.5 : 0.0;
                d.pbc_v[d.npbc][q] = q == k ? double(L[k]) - 2.0 : 0.0;
            }
            ++d.npbc;
        }
    }
    // particles of the elements (DEM::compositeProperties, elmt::generateParticles;
    // DEM.cpp:404-433, elmt.cpp:122-137): element k owns particles efirst[k] ..
    // efirst[k+1]-1 at its prototype's positions (radius units)
    std::vector<int> esz(E, 1), efirst(E + 1, 0);
    for (int k = 0; k < E; ++k) {
        if (e->size) esz[k] = e->size[k];
        if (esz[k] < 1 || esz[k] > 4) return seterr(HB_ERR_ARG, "element %d: size %d (1..4 spheres)", k, esz[k]);
        efirst[k + 1] = efirst[k] + esz[k];
    }
    const int Pn = efirst[E];
    d.P = Pn;
    d.gen = (d.npbc > 0 || Pn != E) ? 1 : 0;
    double proto[5][4][3] = {};
    proto[2][0][0] = 0.5; proto[2][1][0] = -0.5;
    proto[3][0][1] = 1.0;
    proto[3][1][0] = -std::sqrt(3.0) / 2; proto[3][1][1] = -1 / 2;  // integer division: 0
    proto[3][2][0] = std::sqrt(3.0) / 2; proto[3][2][1] = -1 / 2;
    proto[4][0][2] = 1.0;
    proto[4][1][1] = 2.0 * std::sqrt(2.0) / 3.0; proto[4][1][2] = -1.0 / 3.0;
    proto[4][2][0] = 2.0 * std::sqrt(6.0) / 6.0; proto[4][2][1] = -2.0 * std::sqrt(2.0) / 6.0; proto[4][2][2] = -1.0 / 3.0;
    proto[4][3][0] = -2.0 * std::sqrt(6.0) / 6.0; proto[4][3][1] = -2.0 * std::sqrt(2.0) / 6.0; proto[4][3][2] = -1.0 / 3.0;
    // element fields, one allocation (elmt.h:53-135)
    const int nfields = DEM_FIELDS;
    int rc;
    if ((rc = dalloc(&d.base, (size_t)nfields * E))) return rc;
    CK(cudaMemset(d.base, 0, sizeof(double) * nfields * E));
    if ((rc = dalloc(&d.alt, 9 * (size_t)E))) return rc;
    CK(cudaMemset(d.alt, 0, sizeof(double) * 9 * E));
    double* p = d.base;
    auto take = [&](int comps) { double* r = p; p += (size_t)comps * E; return r; };
    for (int k = 0; k < 6; ++k) d.x[k] = take(3);
    for (int k = 0; k < 6; ++k) d.xp[k] = take(3);
    for (int k = 0; k < 6; ++k) d.w[k] = take(3);
    for (int k = 0; k < 6; ++k) d.wp[k] = take(3);
    for (int k = 0; k < 6; ++k) d.q[k] = take(4);
    for (int k = 0; k < 6; ++k) d.qp[k] = take(4);
    d.wG = take(3); d.wL = take(3); d.wpG = take(3); d.wpL = take(3);
    d.FH = take(3); d.MH = take(3); d.FP = take(3); d.FW = take(3); d.MP = take(3); d.MW = take(3);
    d.fvol = take(1); d.m = take(1); d.I = take(3); d.rad = take(1);
    // host-side element init (elmt.cpp:13-61)
    std::vector<double> m(E), I(3 * E), q0(4 * E), w0(3 * E, 0.0), x1(3 * E, 0.0);
    double maxRad = 0.0;
    for (int k = 0; k < E; ++k) {
        const double r = e->radius[k];
        maxRad = std::max(maxRad, r);
        const double sm = 4.0 / 3.0 * P.density * M_PI * r * r * r;
        const int sz = esz[k];
        m[k] = sz * sm;
        // inertia of the spheres plus their transport terms (elmt.cpp:64-71)
        const double iv = sz * 2.0 / 5.0 * sm * r * r;
        for (int q = 0; q < 3; ++q) I[q * E + k] = 1.0 * iv;
        for (int n = 0; n < sz; ++n) {
            const double* v = proto[sz][n];
            const double t[3] = {v[1] * v[1] + v[2] * v[2], v[2] * v[2] + v[0] * v[0], v[0] * v[0] + v[1] * v[1]};
            for (int q = 0; q < 3; ++q) I[q * E + k] += t[q] * (sm * r * r);
        }
        if (e->q0) for (int q = 0; q < 4; ++q) q0[q * E + k] = e->q0[q * E + k];
        else { q0[k] = 1.0; q0[E + k] = q0[2 * E + k] = q0[3 * E + k] = 0.0; }
        if (e->w0) for (int q = 0; q < 3; ++q) w0[q * E + k] = e->w0[q * E + k];
        if (e->x1) for (int q = 0; q < 3; ++q) x1[q * E + k] = e->x1[q * E + k];
    }
    CK(cudaMemcpy(d.x[0], e->x0, sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.xp[0], e->x0, sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.x[1], x1.data(), sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.xp[1], x1.data(), sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    for (double* dst : {d.w[0], d.wG, d.wL, d.wpG, d.wpL})
        CK(cudaMemcpy(dst, w0.data(), sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.q[0], q0.data(), sizeof(double) * 4 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.qp[0], q0.data(), sizeof(double) * 4 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.m, m.data(), sizeof(double) * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.I, I.data(), sizeof(double) * 3 * E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.rad, e->radius, sizeof(double) * E, cudaMemcpyHostToDevice));
    {  // FP32 copy read by the reduced-precision lattice kernel
        std::vector<float> pf(12 * (size_t)E, 0.0f);  // per particle: centre, velocity, spin, pad
        for (int k = 0; k < E; ++k)
            for (int q = 0; q < 3; ++q) {
                pf[12 * (size_t)k + q] = (float)e->x0[q * E + k];
                pf[12 * (size_t)k + 3 + q] = (float)x1[q * E + k];
                pf[12 * (size_t)k + 6 + q] = (float)w0[q * E + k];
            }
        if ((rc = dalloc(&d.pf, 12 * (size_t)E))) return rc;
        std::vector<int> plain(E);
        for (int k = 0; k < E; ++k) {
            const bool ident = q0[k] == 1.0 && q0[E + k] == 0.0 && q0[2 * E + k] == 0.0 && q0[3 * E + k] == 0.0;
            plain[k] = ident && esz[k] == 1 ? 1 : 0;  // q1 (quaternion rate) is zero for every uploaded element
        }
        if ((rc = dalloc(&d.plain, E))) return rc;
        CK(cudaMemcpy(d.plain, plain.data(), sizeof(int) * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.pf, pf.data(), sizeof(float) * pf.size(), cudaMemcpyHostToDevice));
    }
    // neighbour-list parameters (DEM.cpp:1270-1312)
    const double demSize[3] = {(double)c->X, (double)c->Y, (double)c->Z};
    for (int k = 0; k < 3; ++k) {
        d.cellWidth[k] = std::min(maxRad * 5.0, demSize[k]);
        d.nCells[k] = (int)std::ceil(demSize[k] / d.cellWidth[k]);
        d.cellWidth[k] = demSize[k] / double(d.nCells[k]);
        d.nCells[k] += 2;
    }
    d.nebrRange = std::max(maxRad * 3.0, 0.5 * std::min(d.cellWidth[0], std::min(d.cellWidth[1], d.cellWidth[2])));
    d.trigger = 0.25 * d.nebrRange;
    d.ncells = d.nCells[0] * d.nCells[1] * d.nCells[2];
    if (d.npbc) {
        // periodicObjects (DEM.cpp:990-1063): an object within 2 nebrRange of a face (pl1
        // tested first) gets one image per face pair, then one per two images of the same
        // object, appended after the uploaded objects
        std::vector<int> gi;
        std::vector<double> gv;
        for (int b = 0; b < d.npbc; ++b) {
            const double* v = d.pbc_v[b];
            const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const double n1[3] = {v[0] / nv, v[1] / nv, v[2] / nv};
            for (int k = 0; k < O0; ++k) {
                const double* x = &ox[3 * k];
                const double ld = n1[0] * (x[0] - d.pbc_p[b][0]) + n1[1] * (x[1] - d.pbc_p[b][1]) + n1[2] * (x[2] - d.pbc_p[b][2]);
                const double rd = (-1.0 * n1[0]) * (x[0] - (d.pbc_p[b][0] + v[0])) + (-1.0 * n1[1]) * (x[1] - (d.pbc_p[b][1] + v[1])) +
                                  (-1.0 * n1[2]) * (x[2] - (d.pbc_p[b][2] + v[2]));
                if (ld < 2.0 * d.nebrRange && ld > 0.0) {
                    gi.push_back(k);
                    for (int q = 0; q < 3; ++q) gv.push_back(v[q]);
                } else if (rd < 2.0 * d.nebrRange && rd > 0.0) {
                    gi.push_back(k);
                    for (int q = 0; q < 3; ++q) gv.push_back(-1.0 * v[q]);
                }
            }
        }
        const size_t ns = gi.size();
        for (size_t g1 = 0; g1 < ns; ++g1)
            for (size_t g2 = g1 + 1; g2 < ns; ++g2)
                if (gi[g1] == gi[g2]) {
                    gi.push_back(gi[g1]);
                    for (int q = 0; q < 3; ++q) gv.push_back(gv[3 * g1 + q] + gv[3 * g2 + q]);
                }
        for (size_t g = 0; g < gi.size(); ++g) {
            for (int q = 0; q < 3; ++q) {
                ox.push_back(ox[3 * gi[g] + q] + gv[3 * g + q]);
                ov.push_back(ov[3 * gi[g] + q]);
            }
            orr.push_back(orr[gi[g]]);
        }
    }
    if (d.gen) {
        // per-particle path: ghost particles (at most one per face pair and one per two of
        // those per particle) and the particle tables
        const size_t Ps = (size_t)Pn;
        d.gcap = d.npbc ? 6 * Pn : 0;
        const size_t S = Ps + d.gcap;
        auto zi = [&](int** p_, size_t n) -> int {
            int r_ = dalloc(p_, n);
            if (!r_) cudaMemset(*p_, 0, sizeof(int) * std::max<size_t>(n, 1));
            return r_;
        };
        auto zd = [&](double** p_, size_t n) -> int {
            int r_ = dalloc(p_, n);
            if (!r_) cudaMemset(*p_, 0, sizeof(double) * std::max<size_t>(n, 1));
            return r_;
        };
        if ((rc = zi(&d.gmeta, 2)) || (rc = zi(&d.gorig, d.gcap)) || (rc = zd(&d.gvec, 3 * (size_t)d.gcap)) ||
            (rc = zi(&d.comp, 6 * Ps)) || (rc = zi(&d.ccnt, Ps)) || (rc = zi(&d.ecomp, 6 * Ps)) ||
            (rc = zi(&d.eccnt, E)) || (rc = zd(&d.px, 3 * S)) || (rc = zi(&d.pkey, S)) ||
            (rc = zi(&d.efirst, (size_t)E + 1)) || (rc = zi(&d.esize, E)) || (rc = zd(&d.proto, 3 * Ps)) ||
            (rc = zd(&d.ppos, 3 * S)) || (rc = zd(&d.pvel, 3 * S)) || (rc = zd(&d.prv, 3 * S)) ||
            (rc = zd(&d.pF, 12 * Ps)) || (rc = zd(&d.pcen, 3 * S)))
            return rc;
        std::vector<int> key(S, 0);
        std::vector<double> pr(3 * Ps, 0.0);
        for (int k = 0; k < E; ++k)
            for (int n = 0; n < esz[k]; ++n) {
                const int q = efirst[k] + n;
                key[q] = k;
                for (int c3 = 0; c3 < 3; ++c3) pr[c3 * Ps + q] = proto[esz[k]][n][c3];
            }
        CK(cudaMemcpy(d.pkey, key.data(), sizeof(int) * S, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.efirst, efirst.data(), sizeof(int) * (E + 1), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.esize, esz.data(), sizeof(int) * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d.proto, pr.data(), sizeof(double) * pr.size(), cudaMemcpyHostToDevice));
        // the FP32 records are per particle (ghosts after the standard ones)
        cudaFree(d.pf);
        d.pf = nullptr;
        if ((rc = dalloc(&d.pf, 12 * S))) return rc;
        CK(cudaMemset(d.pf, 0, sizeof(float) * 12 * S));
    }
    if ((rc = upload_objects())) return rc;
    const size_t Pl = (size_t)(d.gen ? Pn : E);  // particles that own candidate lists
    const size_t S = Pl + d.gcap;
    if ((rc = dalloc(&d.cell_of, S)) || (rc = dalloc(&d.cell_cnt, d.ncells)) || (rc = dalloc(&d.cell_start, d.ncells + 1)) ||
        (rc = dalloc(&d.cell_fill, d.ncells)) || (rc = dalloc(&d.cell_items, S)) ||
        (rc = dalloc(&d.nbr, Pl * (size_t)d.nbr_cap)) || (rc = dalloc(&d.nbr_cnt, Pl)) || (rc = dalloc(&d.wall_of, Pl)) ||
        (rc = dalloc(&d.obj, Pl * OBJ_CAP)) || (rc = dalloc(&d.obj_cnt, Pl)) || (rc = dalloc(&d.scal, 8)) ||
        (rc = dalloc(&d.contacts, 1)) || (rc = dalloc(&d.partial, hb::PARTIAL_CAP)) || (rc = dalloc(&d.done, 1)) ||
        (rc = dalloc(&d.wrec, 7 * Pl)) || (rc = dalloc(&d.orec, 7 * Pl * OBJ_CAP)) ||
        (rc = dalloc(&d.cyl_of, Pl)) ||
        (rc = dalloc(&d.react, (size_t)3 * (MAX_WALLS + d.O))) ||
        (!d.gen && (rc = dalloc(&d.npc, 4 * Pl * (size_t)d.nbr_cap))))
        return rc;
    CK(cudaMemset(d.react, 0, sizeof(double) * 3 * (MAX_WALLS + d.O)));
    CK(cudaMemset(d.wrec, 0, sizeof(double) * 7 * Pl));
    CK(cudaMemset(d.cyl_of, 0xFF, sizeof(int) * Pl));
    CK(cudaMemset(d.orec, 0, sizeof(double) * 7 * Pl * OBJ_CAP));
    const double scal0[8] = {0.5 * d.nebrRange, 1.0, 0, 0, 0, 0, 0, 0};  // maxDisp, rebuild
    CK(cudaMemcpy(d.scal, scal0, sizeof(scal0), cudaMemcpyHostToDevice));
    CK(cudaMemset(d.contacts, 0, sizeof(int)));
    CK(cudaMemset(d.done, 0, sizeof(unsigned int)));
    CK(cudaMemset(d.nbr_cnt, 0, sizeof(int) * Pl));
    CK(cudaMemset(d.obj_cnt, 0, sizeof(int) * Pl));
    return HB_OK;
}

}  // namespace hb

using namespace hb;

static int build_graph(hb_ctx* c);

// the element force sums of a lattice step are completed by the next cycle (or a
// download) -- except with moving bounce-back in FP64, whose force pass writes them
static bool sums_lag(const hb_ctx* c) {
    return !(c->P.coupling == HB_MOVING_BB && c->P.precision == HB_FP64);
}

extern "C" {

const char* hb_last_error(void) { return g_err.c_str(); }

int hb_create(const hb_params* params, hb_ctx** out) {
    if (!params || !out) return seterr(HB_ERR_ARG, "null argument");
    int rc = check_params(params);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return seterr(HB_ERR_CUDA, "no CUDA device");
    hb_ctx* c = new hb_ctx();
    c->P = *params;
    c->X = params->lb_size[0];
    c->Y = params->lb_size[1];
    c->Z = params->lb_size[2];
    c->N = (long long)c->X * c->Y * c->Z;
    CK(cudaGetDevice(&c->dev));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    const long long N = c->N;
    c->sz = params->precision == HB_FP64 ? 8 : (params->precision == HB_FP32 ? 4 : 2);
    const size_t tsz = params->precision == HB_FP64 ? 8 : 4;
    if ((rc = dalloc(&c->ntype, N)) || (rc = dalloc(&c->solid, N)) || (rc = dalloc((uint8_t**)&c->fA, 19 * N * c->sz)) ||
        (rc = dalloc((uint8_t**)&c->fB, 19 * N * c->sz)) || (rc = dalloc(&c->mode, 1)) ||
        (rc = dalloc(&c->rho, N)) || (rc = dalloc(&c->u, 3 * N)) || (rc = dalloc(&c->hf, 3 * N)) ||
        (rc = dalloc(&c->mass, N)) || (rc = dalloc(&c->status, STATUS_WORDS)) ||
        (rc = dalloc(&c->wall_force, MAX_WALLS * 3 + 1))) {
        hb_destroy(c);
        return rc;
    }
    if (params->non_newtonian || params->turbulence)
        if ((rc = dalloc((uint8_t**)&c->visc, N * tsz))) { hb_destroy(c); return rc; }
    if (params->precision != HB_FP64)
        if ((rc = dalloc(&c->lmask, N))) { hb_destroy(c); return rc; }
    CK(cudaMemset(c->mode, 0, sizeof(int)));
    CK(cudaMemset(c->status, 0, sizeof(int) * STATUS_WORDS));
    // node fields start defined: a phase may read a node's value before the lattice first
    // writes it (the element-force reduction of the first cycle reads the forcing term)
    CK(cudaMemset(c->rho, 0, sizeof(double) * N));
    CK(cudaMemset(c->u, 0, sizeof(double) * 3 * N));
    CK(cudaMemset(c->hf, 0, sizeof(double) * 3 * N));
    CK(cudaMemset(c->mass, 0, sizeof(double) * N));
    CK(cudaMemset(c->wall_force, 0, sizeof(double) * (MAX_WALLS * 3 + 1)));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    *out = c;
    return HB_OK;
}

int hb_destroy(hb_ctx* c) {
    if (!c) return HB_OK;
    hb::adjoint_free(c);
    for (int k = 0; k < 2; ++k)
        if (c->gexec[k]) cudaGraphExecDestroy(c->gexec[k]);
    if (c->graph) cudaGraphDestroy(c->graph);
    if (c->graph2) cudaGraphDestroy(c->graph2);
    void* ptrs[] = {c->ntype, c->lmask, c->solid, c->fA, c->fB, c->mode, c->rho, c->u, c->hf, c->mass,
                    c->visc, c->dv, c->hacc, c->status, c->wall_part, c->wall_force, c->fs_force, c->fs_mass2,
                    c->fs_scal, c->fs_flag, c->fs_first, c->fs_parent, c->lb_force, c->d_stage, c->d.pf, c->d.plain,
                    c->d.base, c->d.alt, c->d.cell_of, c->d.cell_cnt, c->d.cell_start, c->d.cell_fill, c->d.cell_items,
                    c->d.nbr, c->d.npc, c->d.nbr_cnt, c->d.wall_of, c->d.obj, c->d.obj_cnt, c->d.scal, c->d.contacts,
                    c->d.partial, c->d.done, c->d.obj_x0, c->d.obj_x1, c->d.obj_r,
                    c->d.claim_list, c->d.claim_cnt, c->d.mask_done, c->d.pop_list, c->d.pop_cnt, c->d.pop_rho, c->d.boxes, c->d.gargs, c->d.wrec, c->d.orec, c->d.react,
                    c->io_linked, c->io_part, c->slip_list, c->slip_val, c->slip_mix, c->fs_ilist,
                    c->curved_list, c->curved_cnt, c->d.cyl_of, c->io_terms, c->d.gmeta, c->d.gorig, c->d.gvec,
                    c->d.comp, c->d.ccnt, c->d.px, c->d.remark, c->d.ecomp, c->d.eccnt, c->d.pkey, c->d.efirst,
                    c->d.esize, c->d.proto, c->d.ppos, c->d.pvel, c->d.prv, c->d.pF, c->d.pcen};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return HB_OK;
}

int hb_set_cylinders(hb_ctx* c, const hb_cylinders* cy) {
    if (!c || !cy) return seterr(HB_ERR_ARG, "null argument");
    if (c->initialized) return seterr(HB_ERR_STATE, "cylinders must be set before hb_init");
    if (cy->count < 0 || cy->count > 8 || (cy->count && (!cy->p1 || !cy->p2 || !cy->radius)))
        return seterr(HB_ERR_ARG, "cylinders: 0..8 with p1, p2, radius");
    c->cyl.clear();
    for (int k = 0; k < cy->count; ++k) {
        hb_cyl_host h = {};
        for (int q = 0; q < 3; ++q) {
            h.p1[q] = cy->p1[3 * k + q];
            h.p2[q] = cy->p2[3 * k + q];
            h.omega[q] = cy->omega ? cy->omega[3 * k + q] : 0.0;
        }
        h.R = cy->radius[k];
        h.moving = cy->moving ? cy->moving[k] : 0;
        if (h.p1[0] == h.p2[0] && h.p1[1] == h.p2[1] && h.p1[2] == h.p2[2]) return seterr(HB_ERR_ARG, "cylinder axis of zero length");
        c->cyl.push_back(h);
    }
    return HB_OK;
}

int hb_init(hb_ctx* c, const hb_elements* e, const hb_objects* o) {
    if (!c) return seterr(HB_ERR_ARG, "null ctx");
    if (!c->cyl.empty() && c->P.free_surface)
        return seterr(HB_ERR_UNSUPPORTED, "cylinders (curved walls) with a free surface are not implemented");
    if (c->cyl.size() > 4 && c->P.dem_solve && e && e->count > 0)
        return seterr(HB_ERR_UNSUPPORTED, "more than 4 cylinders with moving particles");
    int rc = dem_init(c, e, o);
    if (rc) return rc;
    const long long N = c->N;
    const bool mbb = c->P.coupling == HB_MOVING_BB && c->d.E > 0;
    if (mbb && (c->d.gen || !c->cyl.empty()))
        return seterr(HB_ERR_UNSUPPORTED,
                      "moving bounce-back coupling takes single spheres without periodic faces or cylinders");
    const size_t tsz = c->P.precision == HB_FP64 ? 8 : 4;
    if (c->d.E > 0) {
        if (c->P.precision == HB_FP64) {
            // direct-forcing term per node: zero until the first lattice step (the first
            // cycle's element sums, before any lattice step, are FHydro = 0 as the
            // reference's element init leaves them)
            if (!c->dv && (rc = dalloc((uint8_t**)&c->dv, 3 * N * tsz))) return rc;
            CK(cudaMemset(c->dv, 0, 3 * N * tsz));
        } else {
            if (!c->hacc && (rc = dalloc(&c->hacc, 7 * (size_t)c->d.E))) return rc;
            CK(cudaMemset(c->hacc, 0, sizeof(unsigned long long) * 7 * c->d.E));
        }
        if (!c->d.claim_list && (rc = dalloc(&c->d.claim_list, 2 * N))) return rc;
        if (!c->d.claim_cnt && (rc = dalloc(&c->d.claim_cnt, 1))) return rc;
        if (!c->d.mask_done && (rc = dalloc(&c->d.mask_done, 1))) return rc;
        CK(cudaMemset(c->d.mask_done, 0, sizeof(unsigned int)));
        if (!c->d.boxes && (rc = dalloc((uint8_t**)&c->d.boxes, ((size_t)c->d.P + c->d.gcap) * 128))) return rc;
        CK(cudaMemset(c->d.claim_cnt, 0, sizeof(int)));
        if (mbb) {
            if (!c->d.pop_list && (rc = dalloc(&c->d.pop_list, N))) return rc;
            if (!c->d.pop_cnt && (rc = dalloc(&c->d.pop_cnt, 1))) return rc;
            if (!c->d.pop_rho && (rc = dalloc(&c->d.pop_rho, N))) return rc;
            CK(cudaMemset(c->d.pop_cnt, 0, sizeof(int)));
        }
        if (c->d.npbc && c->P.lb_solve && !c->d.remark) {
            if ((rc = dalloc(&c->d.remark, N))) return rc;
            CK(cudaMemset(c->d.remark, 0, sizeof(uint32_t) * N));
        }
    }
    if (!c->wall_part) {
        const long long grid = (long long)ceil_div(c->X, c->X <= 64 ? 64 : (c->X <= 128 ? 128 : 256)) * (c->Y - 2) * (c->Z - 2);
        if ((rc = dalloc(&c->wall_part, (size_t)grid * (MAX_WALLS * 3 + 1)))) return rc;
    }
    if (!c->fs_force) {
        if ((rc = dalloc(&c->fs_force, 3))) return rc;
    }
    if (!c->lb_force) {
        if ((rc = dalloc(&c->lb_force, 5))) return rc;
        c->lb_force_f = reinterpret_cast<float*>(c->lb_force + 3);
    }
    {
        const float ff[3] = {c->P.force_field ? (float)c->P.lbF[0] : 0.f, c->P.force_field ? (float)c->P.lbF[1] : 0.f,
                             c->P.force_field ? (float)c->P.lbF[2] : 0.f};
        CK(cudaMemcpy(c->lb_force_f, ff, sizeof(ff), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(c->fs_force, c->P.lbF, sizeof(double) * 3, cudaMemcpyHostToDevice));
    {
        const double z[3] = {0.0, 0.0, 0.0};
        CK(cudaMemcpy(c->lb_force, c->P.force_field ? c->P.lbF : z, sizeof(double) * 3, cudaMemcpyHostToDevice));
    }
    c->cur = 0;
    c->reduce_pending = false;
    c->steps = 0;
    c->dem_stepped = false;
    if (launch_ghosts_init(c)) return seterr(HB_ERR_CUDA, "particles: %s", cudaGetErrorString(cudaGetLastError()));
    if (launch_init_lattice(c, e && c->d.E ? c->d.x[0] : nullptr, c->d.E ? c->d.rad : nullptr, c->d.E,
                            c->d.obj_x0, c->d.obj_r, c->d.O))
        return seterr(HB_ERR_CUDA, "lattice init: %s", cudaGetErrorString(cudaGetLastError()));
    if (slip_init(c)) return seterr(HB_ERR_CUDA, "slip-wall list: %s", cudaGetErrorString(cudaGetLastError()));
    if (curved_init(c)) return seterr(HB_ERR_CUDA, "curved-wall list: %s", cudaGetErrorString(cudaGetLastError()));
    // count dynamic-wall nodes (the context stream does not synchronise with the default
    // stream: wait for the init kernels first)
    {
        std::vector<uint8_t> t(N);
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(t.data(), c->ntype, N, cudaMemcpyDeviceToHost));
        c->has_dynwall = false;
        for (long long i = 0; i < N; ++i)
            if ((t[i] & HB_TYPE_MASK) == HB_T_DYNWALL) { c->has_dynwall = true; break; }
    }
    if (c->P.free_surface) {
        if ((rc = fs_init(c))) return rc;
    }
    // the reference builds the neighbour table at init (DEM.cpp:253-257) and, because
    // maxDisp starts at 0.5 nebrRange, again at the first substep; only the second is
    // ever used, so the first trigger evaluation sets the rebuild flag here
    if (c->d.E > 0) launch_dem_first_predict(c);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    if (dem_args_upload(c)) return seterr(HB_ERR_CUDA, "DEM parameter upload: %s", cudaGetErrorString(cudaGetLastError()));
    c->initialized = true;
    if ((rc = build_graph(c))) return rc;
    return HB_OK;
}

int hb_upload_lattice(hb_ctx* c, const uint8_t* type, const uint8_t* inside, const uint32_t* solid,
                      const double* f, const double* n, const double* u, const double* mass, const double* visc) {
    if (!c || !type || !inside || !solid || !n || !u || !mass) return seterr(HB_ERR_ARG, "null argument");
    if (!c->initialized) return seterr(HB_ERR_STATE, "hb_init must run first");
    if (launch_upload_lattice(c, type, inside, solid, f, n, u, mass, visc))
        return seterr(HB_ERR_CUDA, "upload: %s", cudaGetErrorString(cudaGetLastError()));
    curved_remark(c);  // the uploaded node bytes carry no velocity-mirror bits
    hb::fs_invalidate(c);  // new node types: the interface list is rebuilt at the next step
    c->mirror_valid = true;  // the node fields are the uploaded ones
    CK(cudaStreamSynchronize(c->stream));
    return HB_OK;
}

}  // extern "C"

static int enqueue_sink_gather(hb_ctx* c);

// one whole cycle on the context stream, starting from population buffer `cur`
static int enqueue_cycle(hb_ctx* c, int cur) {
    const bool dem = c->P.dem_solve && c->d.E > 0;
    // R (element forces of the previous lattice step) + DEM substeps + coupling masks
    if (dem && launch_cycle_coop(c, 1, 1, c->P.lb_solve ? 1 : 0)) return -1;
    if (!c->P.lb_solve) return 0;
    if (dem) launch_couple(c, false, cur);
    if (c->P.free_surface) launch_fs_step(c, cur);
    launch_lb_step(c, cur);
    if (c->has_dynwall) launch_lb_wallforce(c, cur);
    if (!c->P.force_field) cudaMemsetAsync(c->fs_force, 0, sizeof(double) * 3, c->stream);
    if (c->sink_on && enqueue_sink_gather(c)) return -1;
    return 0;
}

static int build_graph(hb_ctx* c) {
    hb::flush_body_force(c);  // the capture takes lbF from the parameters
    for (int k = 0; k < 2; ++k) {
        if (c->gexec[k]) { cudaGraphExecDestroy(c->gexec[k]); c->gexec[k] = nullptr; }
    }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
    if (c->graph2) { cudaGraphDestroy(c->graph2); c->graph2 = nullptr; }
    for (int k = 0; k < 2; ++k) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_cycle(c, k);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc || e != cudaSuccess)
            return seterr(HB_ERR_CUDA, "cycle capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : cudaGetLastError()));
        CK(cudaGraphInstantiate(&c->gexec[k], g, 0));
        if (k == 0) c->graph = g; else c->graph2 = g;
        c->mask_node[k] = hb::find_mask_node(g);
    }
    size_t nn = 0;
    CK(cudaGraphGetNodes(c->graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(c->graph, nodes.data(), &nn));
    int k = 0;
    for (auto& nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    c->kernels_per_cycle = k;
    return HB_OK;
}

namespace hb {
// concatenation of up to 11 element fields into one staging block (one copy to the host)
constexpr int STAGE_DOUBLES_PER_ELEMENT = 35;
struct GatherArgs {
    const double* src[11];
    double* dst[11];  // per-field destinations (mapped host memory), or all null: the staging block
    long long off[12];
    int hsum[11];  // >= 0: the field is the element sums' component hsum.. (FHydro 0, MHydro 3,
                   // fluidVolume 6) converted from the fixed-point accumulators on the fly
    int n, E;
    const unsigned long long* hacc;
};

__global__ void k_gather(GatherArgs g, double* dst) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.off[g.n]) return;
    int k = 0;
    while (k + 1 < g.n && t >= g.off[k + 1]) ++k;
    const long long r = t - g.off[k];
    double v;
    if (g.hsum[k] >= 0) {  // (r / E) selects the component, as in convert_sums
        const long long comp = r / g.E, p = r - comp * g.E;
        v = (double)(long long)g.hacc[(g.hsum[k] + comp) * g.E + p] * HACC_INV;
    } else {
        v = g.src[k][r];
    }
    if (g.dst[k]) g.dst[k][r] = v;  // straight into the caller's mapped host array
    else dst[t] = v;
}

// lbF and its FP32 copy from kernel arguments (stream-ordered, no host staging)
__global__ void k_set_force(double* f, double fx, double fy, double fz) {
    f[0] = fx; f[1] = fy; f[2] = fz;
    float* ff = reinterpret_cast<float*>(f + 3);
    ff[0] = (float)fx; ff[1] = (float)fy; ff[2] = (float)fz; ff[3] = 0.0f;
}

// paths outside the cycle graphs (single phases, checkpoints, a new capture) read
// lb_force itself: write it now when the graphs hold a newer lbF
void flush_body_force(hb_ctx* c) {
    if (!c->force_dirty) return;
    k_set_force<<<1, 1, 0, c->stream>>>(c->lb_force, c->P.lbF[0], c->P.lbF[1], c->P.lbF[2]);
    c->force_dirty = false;
}
}  // namespace hb

static int run_cycles(hb_ctx* c, int n, bool last_mirror) {
    for (int s = 0; s < n; ++s) {
        const int m = (last_mirror && s == n - 1) ? 1 : 0;
        if (m != c->mode_val) {
            CK(cudaMemsetAsync(c->mode, m, sizeof(int), c->stream));
            c->mode_val = m;
        }
        CK(cudaGraphLaunch(c->gexec[c->cur], c->stream));
        c->force_dirty = false;  // the graph's mask kernel wrote lb_force
        if (c->P.dem_solve && c->d.E > 0) c->dem_stepped = true;
        if (c->P.lb_solve) {
            c->cur ^= 1;
            c->reduce_pending = sums_lag(c);  // the sums lag the lattice step
        }
        ++c->steps;
    }
    if (n > 0 && c->P.lb_solve) c->mirror_valid = last_mirror;
    return HB_OK;
}

static int need_mirror(const hb_ctx* c) {
    if (c->mirror_valid || !c->P.lb_solve) return HB_OK;
    return seterr(HB_ERR_STATE, "the node fields (rho, u, hydroForce) of the last step were not written: the last "
                  "cycles ran with hb_set_lattice_mirror(ctx, 0) or through the timing entry points; run a cycle "
                  "with the mirror on first");
}

extern "C" {

int hb_set_lattice_mirror(hb_ctx* c, int32_t on) {
    if (!c) return seterr(HB_ERR_ARG, "null ctx");
    c->mirror = on != 0;
    return HB_OK;
}

int hb_dem_step(hb_ctx* c) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (c->P.dem_solve && c->d.E > 0) {
        if (launch_cycle_coop(c, 1, 1, 0)) return seterr(HB_ERR_CUDA, "DEM launch: %s", cudaGetErrorString(cudaGetLastError()));
        c->reduce_pending = false;
        c->dem_stepped = true;
    }
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_fs_step(hb_ctx* c) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    hb::flush_body_force(c);
    if (c->P.free_surface) launch_fs_step(c, c->cur);
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_coupling_step(hb_ctx* c) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (c->P.dem_solve && c->d.E > 0) {
        launch_couple(c, true, c->cur);
    }
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_lb_step(hb_ctx* c) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    hb::flush_body_force(c);
    CK(cudaMemsetAsync(c->mode, 1, sizeof(int), c->stream));
    c->mode_val = 1;
    c->mirror_valid = true;
    launch_lb_step(c, c->cur);
    if (c->has_dynwall) launch_lb_wallforce(c, c->cur);
    if (!c->P.force_field) CK(cudaMemsetAsync(c->fs_force, 0, sizeof(double) * 3, c->stream));
    c->cur ^= 1;
    c->reduce_pending = sums_lag(c);  // the sums lag the lattice step
    ++c->steps;
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_cycle(hb_ctx* c, int32_t nsteps) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (nsteps < 0) return seterr(HB_ERR_ARG, "nsteps < 0");
    int rc = run_cycles(c, nsteps, c->mirror);
    if (rc) return rc;
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_get_params(hb_ctx* c, hb_params* out, int32_t* elements, int32_t* objects) {
    if (!c) return seterr(HB_ERR_ARG, "null ctx");
    if (out) *out = c->P;
    if (elements) *elements = c->d.E;
    if (objects) *objects = c->d.O;
    return HB_OK;
}

int hb_set_body_force(hb_ctx* c, const double* force) {
    if (!c || !force || !c->initialized) return seterr(HB_ERR_ARG, "null argument or not initialised");
    for (int k = 0; k < 3; ++k) c->P.lbF[k] = force[k];
    if (!c->P.force_field) return HB_OK;
    if (c->mask_node[0] && c->mask_node[1]) {
        // the cycle graphs' mask kernel writes it before the lattice step: no launch of its
        // own between two cycles
        if (hb::update_mask_force(c)) return seterr(HB_ERR_CUDA, "graph update: %s", cudaGetErrorString(cudaGetLastError()));
        c->force_dirty = true;
        return HB_OK;
    }
    hb::k_set_force<<<1, 1, 0, c->stream>>>(c->lb_force, force[0], force[1], force[2]);
    CK(cudaGetLastError());
    return HB_OK;
}

int hb_synchronize(hb_ctx* c) {
    if (!c) return seterr(HB_ERR_ARG, "null ctx");
    CK(cudaStreamSynchronize(c->stream));
    int st[STATUS_WORDS];
    CK(cudaMemcpy(st, c->status, sizeof(st), cudaMemcpyDeviceToHost));
    if (st[1]) return seterr(HB_ERR_UNSUPPORTED, "TYPE ERROR: an active node links to an unsupported node type");
    // status word 2: 1 candidate list full, 2 particle outside the cell grid, 4 object
    // list full, 8 interface list full
    if (st[2])
        return seterr(HB_ERR_CAPACITY, "list capacity exceeded (code %d:%s%s%s%s; limits %d candidates per particle, "
                      "%d objects per particle, %lld interface cells)",
                      st[2], (st[2] & 1) ? " candidate list full" : "",
                      (st[2] & 2) ? " a particle outside the DEM cell grid" : "",
                      (st[2] & 4) ? " object list full" : "", (st[2] & 8) ? " interface list full" : "",
                      c->d.nbr_cap, OBJ_CAP, (long long)c->fs_icap);
    // status word 0: NaN/Inf density or velocity seen by a lattice kernel (the reference
    // has no such check; its state would carry the NaN on)
    if (st[0]) return seterr(HB_ERR_NUMERIC, "NaN or Inf in a node's density or velocity");
    return HB_OK;
}

int hb_download_lattice(hb_ctx* c, uint8_t* type, uint8_t* inside, uint32_t* solid, double* f, double* n,
                        double* u, double* mass, double* visc, double* hydro_force) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if ((n || u || hydro_force) && need_mirror(c)) return HB_ERR_STATE;
    CK(cudaStreamSynchronize(c->stream));
    const long long N = c->N;
    if (type || inside) {
        std::vector<uint8_t> t(N);
        CK(cudaMemcpy(t.data(), c->ntype, N, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < N; ++i) {
            if (type) type[i] = t[i] & HB_TYPE_MASK;
            if (inside) inside[i] = (t[i] & HB_INSIDE) ? 1 : 0;
        }
    }
    if (solid) CK(cudaMemcpy(solid, c->solid, sizeof(uint32_t) * N, cudaMemcpyDeviceToHost));
    if (f) {
        double* df = nullptr;
        int rc = dalloc(&df, 19 * N);
        if (rc) return rc;
        launch_download_lattice(c, df, c->cur);
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(f, df, sizeof(double) * 19 * N, cudaMemcpyDeviceToHost));
        cudaFree(df);
    }
    if (n) CK(cudaMemcpy(n, c->rho, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (u) CK(cudaMemcpy(u, c->u, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    if (mass) CK(cudaMemcpy(mass, c->mass, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (hydro_force) CK(cudaMemcpy(hydro_force, c->hf, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    if (visc) {
        if (!c->visc) {
            for (long long i = 0; i < N; ++i) visc[i] = c->P.init_visc;
        } else if (c->P.precision == HB_FP64) {
            CK(cudaMemcpy(visc, c->visc, sizeof(double) * N, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> v(N);
            CK(cudaMemcpy(v.data(), c->visc, sizeof(float) * N, cudaMemcpyDeviceToHost));
            for (long long i = 0; i < N; ++i) visc[i] = v[i];
        }
    }
    return HB_OK;
}

}  // extern "C"

// Queues, on the context stream behind the steps already issued, the element-force
// conversion of the last lattice step (LB.cpp:1851-1919) where it is pending and one
// gather of the requested fields into the device staging block.  With the FP32/FP16
// lattice the element sums are read from their fixed-point accumulators inside the
// gather (the next cycle converts them itself); the FP64 form reduces them first.
// items[k].dst non-null selects field k; *g receives the staging offsets.
namespace {
struct ElemItem {
    double* dst;
    double* src;
    int comps;
    int hsum;
};
constexpr int kElemItems = 11;

int ensure_stage(hb_ctx* c);

int enqueue_element_gather(hb_ctx* c, double* const dst[kElemItems], ElemItem items[kElemItems], hb::GatherArgs* g,
                           double* const* alias = nullptr) {
    const int E = c->d.E;
    const bool inline_sums = c->reduce_pending && c->hacc;
    if (c->reduce_pending && !c->hacc) launch_couple_reduce(c);
    const ElemItem all[kElemItems] = {
        {dst[0], c->d.x[0], 3, -1}, {dst[1], c->d.x[1], 3, -1}, {dst[2], c->d.wG, 3, -1}, {dst[3], c->d.q[0], 4, -1},
        {dst[4], c->d.FH, 3, inline_sums ? 0 : -1}, {dst[5], c->d.MH, 3, inline_sums ? 3 : -1},
        {dst[6], c->d.FP, 3, -1}, {dst[7], c->d.FW, 3, -1}, {dst[8], c->d.MP, 3, -1},
        {dst[9], c->d.MW, 3, -1}, {dst[10], c->d.fvol, 1, inline_sums ? 6 : -1}};
    for (int k = 0; k < kElemItems; ++k) items[k] = all[k];
    int rc = ensure_stage(c);
    if (rc) return rc;
    *g = hb::GatherArgs{};
    g->E = E;
    g->hacc = c->hacc;
    for (int k = 0; k < kElemItems; ++k)
        if (items[k].dst) {
            g->src[g->n] = items[k].src;
            g->dst[g->n] = alias ? alias[k] : nullptr;
            g->hsum[g->n] = items[k].hsum;
            g->off[g->n + 1] = g->off[g->n] + (long long)items[k].comps * E;
            ++g->n;
        }
    if (g->n == 0) return HB_OK;
    const long long total = g->off[g->n];
    hb::k_gather<<<(unsigned)ceil_div(total, 256), 256, 0, c->stream>>>(*g, c->d_stage);
    CK(cudaGetLastError());
    return HB_OK;
}

int ensure_stage(hb_ctx* c) {
    if (c->d_stage) return HB_OK;
    const int E = c->d.E;
    int rc = dalloc(&c->d_stage, (size_t)hb::STAGE_DOUBLES_PER_ELEMENT * E);
    if (rc) return rc;
    CK(cudaMallocHost((void**)&c->h_stage, sizeof(double) * hb::STAGE_DOUBLES_PER_ELEMENT * E));
    return HB_OK;
}

// device address of a host array the GPU can write directly (page-locked and mapped, as
// hb_host_register makes it), or null
double* mapped_alias(double* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // an unregistered pointer is not an error here
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? static_cast<double*>(at.devicePointer) : nullptr;
}
}  // namespace

// The element sink at the end of a captured cycle: the lattice step's element sums are
// pending there (FP32/FP16 forms read them from the fixed-point accumulators, the FP64
// form reduces them first, as a download would).
static int enqueue_sink_gather(hb_ctx* c) {
    const bool pending = c->reduce_pending;
    c->reduce_pending = c->P.lb_solve && sums_lag(c);
    ElemItem items[kElemItems];
    hb::GatherArgs g;
    const int rc = enqueue_element_gather(c, c->sink, items, &g, c->sink);
    c->reduce_pending = pending;
    return rc;
}

extern "C" {

int hb_set_element_sink(hb_ctx* c, double* x0, double* x1, double* w, double* q0, double* fhydro, double* mhydro,
                        double* fparticle, double* fwall, double* mparticle, double* mwall, double* fluid_volume) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    double* const dst[kElemItems] = {x0, x1, w, q0, fhydro, mhydro, fparticle, fwall, mparticle, mwall, fluid_volume};
    double* alias[kElemItems] = {};
    bool any = false;
    for (int k = 0; k < kElemItems; ++k) {
        if (!dst[k]) continue;
        if (!(alias[k] = mapped_alias(dst[k])))
            return seterr(HB_ERR_ARG, "sink array %d is not page-locked and mapped (hb_host_register)", k);
        any = true;
    }
    if (any && c->d.E == 0) return seterr(HB_ERR_STATE, "no elements");
    if (any) {
        int rc = ensure_stage(c);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < kElemItems; ++k) c->sink[k] = alias[k];
    c->sink_on = any;
    return build_graph(c);
}

int hb_download_elements(hb_ctx* c, double* x0, double* x1, double* w, double* q0, double* fhydro, double* mhydro,
                         double* fparticle, double* fwall, double* mparticle, double* mwall, double* fluid_volume) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (c->d.E == 0) return HB_OK;
    double* const dst[kElemItems] = {x0, x1, w, q0, fhydro, mhydro, fparticle, fwall, mparticle, mwall, fluid_volume};
    ElemItem items[kElemItems];
    hb::GatherArgs g;
    int rc = enqueue_element_gather(c, dst, items, &g);
    if (rc || g.n == 0) return rc;
    // one copy of the whole staging block into the library's pinned block, then host copies
    CK(cudaMemcpyAsync(c->h_stage, c->d_stage, sizeof(double) * g.off[g.n], cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int k = 0;
    for (auto& it : items)
        if (it.dst) {
            memcpy(it.dst, c->h_stage + g.off[k], sizeof(double) * (g.off[k + 1] - g.off[k]));
            ++k;
        }
    return HB_OK;
}

int hb_download_elements_async(hb_ctx* c, double* x0, double* x1, double* w, double* q0, double* fhydro,
                               double* mhydro, double* fparticle, double* fwall, double* mparticle, double* mwall,
                               double* fluid_volume) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (c->d.E == 0) return HB_OK;
    double* const dst[kElemItems] = {x0, x1, w, q0, fhydro, mhydro, fparticle, fwall, mparticle, mwall, fluid_volume};
    // page-locked, mapped arrays: the gather kernel writes them directly (no copy)
    double* alias[kElemItems] = {};
    bool mapped = true;
    for (int k = 0; k < kElemItems; ++k)
        if (dst[k] && !(alias[k] = mapped_alias(dst[k]))) mapped = false;
    ElemItem items[kElemItems];
    hb::GatherArgs g;
    if (mapped) return enqueue_element_gather(c, dst, items, &g, alias);
    int rc = enqueue_element_gather(c, dst, items, &g);
    if (rc || g.n == 0) return rc;
    // one copy per field straight into the caller's arrays, ordered behind the gather; the
    // next gather into the staging block is ordered behind these copies on the same stream
    int k = 0;
    for (auto& it : items)
        if (it.dst) {
            CK(cudaMemcpyAsync(it.dst, c->d_stage + g.off[k], sizeof(double) * (g.off[k + 1] - g.off[k]),
                               cudaMemcpyDeviceToHost, c->stream));
            ++k;
        }
    return HB_OK;
}

int hb_host_register(void* p, size_t bytes) {
    if (!p || bytes == 0) return seterr(HB_ERR_ARG, "null pointer or zero size");
    CK(cudaHostRegister(p, bytes, cudaHostRegisterMapped));
    return HB_OK;
}

int hb_host_unregister(void* p) {
    if (!p) return seterr(HB_ERR_ARG, "null pointer");
    CK(cudaHostUnregister(p));
    return HB_OK;
}

int hb_download_pairs(hb_ctx* c, uint32_t* pairs, int64_t capacity, int64_t* count) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    CK(cudaStreamSynchronize(c->stream));
    const int E = c->d.P;  // particles (standard ones own the lists)
    std::vector<uint32_t> out;
    if (E > 0) {
        const size_t cap = (size_t)c->d.nbr_cap;
        std::vector<int> nb((size_t)E * cap), cnt(E);
        CK(cudaMemcpy(nb.data(), c->d.nbr, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(cnt.data(), c->d.nbr_cnt, sizeof(int) * E, cudaMemcpyDeviceToHost));
        for (int i = 0; i < E; ++i) {
            std::vector<int> js(nb.begin() + (size_t)i * cap, nb.begin() + (size_t)i * cap + cnt[i]);
            std::sort(js.begin(), js.end());
            for (int j : js)
                if (j > i) { out.push_back((uint32_t)i); out.push_back((uint32_t)j); }
        }
    }
    const int64_t np = (int64_t)out.size() / 2;
    if (count) *count = np;
    if (pairs) memcpy(pairs, out.data(), sizeof(uint32_t) * 2 * std::min(np, capacity));
    return HB_OK;
}

int hb_download_ghosts(hb_ctx* c, uint32_t* origin, double* shift, int64_t capacity, int64_t* count) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    CK(cudaStreamSynchronize(c->stream));
    int G = 0;
    if (c->d.npbc && c->d.E) CK(cudaMemcpy(&G, c->d.gmeta, sizeof(int), cudaMemcpyDeviceToHost));
    if (count) *count = G;
    const int64_t n = std::min<int64_t>(G, capacity);
    if (n <= 0) return HB_OK;
    std::vector<int> o(n);
    std::vector<double> v(3 * (size_t)c->d.gcap);
    CK(cudaMemcpy(o.data(), c->d.gorig, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v.data(), c->d.gvec, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    for (int64_t g = 0; g < n; ++g) {
        if (origin) origin[g] = (uint32_t)o[g];
        if (shift)
            for (int q = 0; q < 3; ++q) shift[3 * g + q] = v[(size_t)q * c->d.gcap + g];
    }
    return HB_OK;
}

int hb_download_interface(hb_ctx* c, uint32_t* cells, int64_t capacity, int64_t* count) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    CK(cudaStreamSynchronize(c->stream));
    const long long N = c->N;
    std::vector<uint8_t> t(N);
    CK(cudaMemcpy(t.data(), c->ntype, N, cudaMemcpyDeviceToHost));
    int64_t k = 0;
    for (long long i = 0; i < N; ++i)
        if ((t[i] & HB_TYPE_MASK) == HB_T_INTERFACE) {
            if (cells && k < capacity) cells[k] = (uint32_t)i;
            ++k;
        }
    if (count) *count = k;
    return HB_OK;
}

int hb_download_walls(hb_ctx* c, double* fhydro, double* fparticle, int32_t* nwalls) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (nwalls) *nwalls = c->d.nw;
    double wr[3 * MAX_WALLS] = {};
    if (fparticle && c->d.react) {
        launch_reactions(c);
        CK(cudaMemcpyAsync(wr, c->d.react, sizeof(wr), cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    double wf[MAX_WALLS * 3 + 1];
    CK(cudaMemcpy(wf, c->wall_force, sizeof(wf), cudaMemcpyDeviceToHost));
    for (int w = 0; w < c->d.nw; ++w)
        for (int k = 0; k < 3; ++k) {
            if (fhydro) fhydro[3 * w + k] = wf[3 * w + k];
            if (fparticle) fparticle[3 * w + k] = wr[3 * w + k];
        }
    return HB_OK;
}

int hb_download_objects(hb_ctx* c, double* fparticle, int32_t* nobjects) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (nobjects) *nobjects = c->d.O;
    if (!fparticle || c->d.O == 0) return HB_OK;
    if (!c->d.react) {  // no moving elements: nothing touches the objects
        memset(fparticle, 0, sizeof(double) * 3 * c->d.O);
        return HB_OK;
    }
    launch_reactions(c);
    CK(cudaMemcpyAsync(fparticle, c->d.react + 3 * MAX_WALLS, sizeof(double) * 3 * c->d.O, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return HB_OK;
}

int hb_get_status(hb_ctx* c, hb_status* s) {
    if (!c || !s) return seterr(HB_ERR_ARG, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    int st[STATUS_WORDS];
    CK(cudaMemcpy(st, c->status, sizeof(st), cudaMemcpyDeviceToHost));
    memset(s, 0, sizeof(*s));
    s->numeric_error = st[0];
    s->capacity_error = st[2];
    s->unsupported_link = st[1];
    if (c->d.E > 0) {
        int k = 0;
        CK(cudaMemcpy(&k, c->d.contacts, sizeof(int), cudaMemcpyDeviceToHost));
        s->contacts = k;
        std::vector<int> cnt(c->d.P);
        CK(cudaMemcpy(cnt.data(), c->d.nbr_cnt, sizeof(int) * c->d.P, cudaMemcpyDeviceToHost));
        int64_t tot = 0;
        for (int v : cnt) tot += v;
        s->pairs = tot / 2;
    }
    if (c->fs_scal) {
        double sc[2];
        CK(cudaMemcpy(sc, c->fs_scal, sizeof(sc), cudaMemcpyDeviceToHost));
        s->mass_surplus = sc[0];
        s->interface_cells = (int64_t)sc[1];
    }
    if (c->P.lb_solve && c->mirror_valid) {  // else active_nodes and total_mass stay 0
        hb_export ex;
        const int rc = hb_export_values(c, &ex);
        if (rc) return rc;
        s->active_nodes = ex.active_nodes;
        s->total_mass = ex.total_fluid_mass;
    }
    return HB_OK;
}

int hb_export_values(hb_ctx* c, hb_export* out) {
    if (!c || !out || !c->initialized) return seterr(HB_ERR_ARG, "null argument or not initialised");
    if (need_mirror(c)) return HB_ERR_STATE;
    if (hb::io_prepare(c)) return seterr(HB_ERR_CUDA, "output mirror: %s", cudaGetErrorString(cudaGetLastError()));
    if (c->reduce_pending) launch_couple_reduce(c);      // FHydro of the last lattice step (LB.cpp:1851-1919)
    if (c->d.E > 0 && c->d.react) hb::launch_reactions(c);  // objects' FParticle of the last substep
    const double* dev = hb::launch_io_export(c);
    double v[32];
    const int ns = hb::io_slot_count();
    CK(cudaMemcpyAsync(v, dev, sizeof(double) * ns, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    memset(out, 0, sizeof(*out));
    // slot order of hb_io.cu (IoSlot)
    out->max_fluid_speed = sqrt(v[0]);
    out->total_fluid_mass = v[1];
    out->active_nodes = (int64_t)v[2];
    out->plastic_nodes = (int64_t)v[3];
    out->plastic_percent = out->active_nodes ? 100.0 * double(out->plastic_nodes) / double(out->active_nodes) : 0.0;
    out->max_particle_speed = sqrt(v[4]);
    out->max_particle_spin = sqrt(v[5]);
    out->collision_force = v[6];
    out->hydraulic_force = v[7];
    out->particle_mass = v[8];
    out->object_force[0] = v[9]; out->object_force[1] = v[10]; out->object_force[2] = v[11];
    // DEM::updateEnergy runs at the end of each substep; before the first, zeros
    if (c->dem_stepped || (c->steps > 0 && c->P.dem_solve && c->d.E > 0)) {
        out->energy_tr_kin = v[12];
        out->energy_rot_kin = v[13];
        out->energy_grav = v[14];
    }
    out->energy_kin = out->energy_rot_kin + out->energy_tr_kin;  // energy::updateTotal (utils.cpp:324-327)
    out->energy_total = out->energy_rot_kin + out->energy_tr_kin + out->energy_grav + 0.0;
    return HB_OK;
}

int hb_vtk_fluid_fields(hb_ctx* c, int8_t* type, double* v, double* pressure, double* dyn_visc, double* mass,
                        uint32_t* solid_index) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (!c->P.lb_solve) return seterr(HB_ERR_STATE, "no lattice (lbSolve = 0)");
    if (need_mirror(c)) return HB_ERR_STATE;
    if (hb::io_prepare(c)) return seterr(HB_ERR_CUDA, "output mirror: %s", cudaGetErrorString(cudaGetLastError()));
    const long long N = c->N;
    // one device block for the requested arrays, one copy per array
    const size_t bytes = (type ? N : 0) + (solid_index ? 4 * N : 0) + 8 * N * ((v ? 3 : 0) + (pressure ? 1 : 0) +
                         (dyn_visc ? 1 : 0) + (mass ? 1 : 0));
    if (bytes == 0) return HB_OK;
    uint8_t* blk = nullptr;
    int rc = dalloc(&blk, bytes + 64);
    if (rc) return rc;
    uint8_t* p = blk;
    auto take = [&](size_t b) { uint8_t* r = p; p += (b + 7) & ~(size_t)7; return r; };
    double* dv = v ? reinterpret_cast<double*>(take(24 * N)) : nullptr;
    double* dp = pressure ? reinterpret_cast<double*>(take(8 * N)) : nullptr;
    double* dvi = dyn_visc ? reinterpret_cast<double*>(take(8 * N)) : nullptr;
    double* dm = mass ? reinterpret_cast<double*>(take(8 * N)) : nullptr;
    uint32_t* ds = solid_index ? reinterpret_cast<uint32_t*>(take(4 * N)) : nullptr;
    int8_t* dt = type ? reinterpret_cast<int8_t*>(take(N)) : nullptr;
    hb::launch_io_pack(c, dt, dv, dp, dvi, dm, ds);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && v) e = cudaMemcpy(v, dv, 24 * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && pressure) e = cudaMemcpy(pressure, dp, 8 * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && dyn_visc) e = cudaMemcpy(dyn_visc, dvi, 8 * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && mass) e = cudaMemcpy(mass, dm, 8 * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && solid_index) e = cudaMemcpy(solid_index, ds, 4 * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && type) e = cudaMemcpy(type, dt, N, cudaMemcpyDeviceToHost);
    cudaFree(blk);
    if (e != cudaSuccess) return seterr(HB_ERR_CUDA, "output mirror copy: %s", cudaGetErrorString(e));
    return HB_OK;
}

int hb_write_vtk_fluid(hb_ctx* c, const char* path) {
    if (!c || !path || !c->initialized) return seterr(HB_ERR_ARG, "null argument or not initialised");
    const long long N = c->N;
    const bool vis = c->P.non_newtonian != 0, fs = c->P.free_surface != 0, dem = c->P.dem_solve != 0;
    std::vector<int8_t> type(N);
    std::vector<double> v(3 * N), pr(N), vi(vis ? N : 0), ms(fs ? N : 0);
    std::vector<uint32_t> so(dem ? N : 0);
    int rc = hb_vtk_fluid_fields(c, type.data(), v.data(), pr.data(), vis ? vi.data() : nullptr,
                                 fs ? ms.data() : nullptr, dem ? so.data() : nullptr);
    if (rc) return rc;
    // IO::exportParaviewFluidOld (IO.cpp:698-831): ASCII image data, default stream
    // formatting; the node loops are formatted in parallel chunks and written in order
    const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    auto section = [&](auto&& one) {
        std::vector<std::string> parts(nth);
        std::vector<std::thread> th;
        for (int t = 0; t < nth; ++t)
            th.emplace_back([&, t] {
                std::ostringstream os;
                os.imbue(std::locale::classic());
                const long long i0 = N * t / nth, i1 = N * (t + 1) / nth;
                for (long long i = i0; i < i1; ++i) one(os, i);
                parts[t] = os.str();
            });
        for (auto& x : th) x.join();
        std::string all;
        for (auto& x : parts) all += x;
        return all;
    };
    std::ofstream f(path, std::ios::binary);
    if (!f) return seterr(HB_ERR_ARG, "cannot open %s", path);
    f.imbue(std::locale::classic());
    const double L = 1.0;
    f << "<VTKFile type=\"ImageData\" version=\"0.1\">\n";
    f << " <ImageData WholeExtent=\"0 " << c->X - 1 << " 0 " << c->Y - 1 << " 0 " << c->Z - 1 << "\" "
      << "Origin=\"0.0 0.0 0.0\" Spacing=\"" << L << " " << L << " " << L << "\">\n";
    f << "  <Piece Extent=\"0 " << c->X - 1 << " 0 " << c->Y - 1 << " 0 " << c->Z - 1 << "\">\n";
    f << "   <PointData>\n";
    f << "    <DataArray type=\"Int8\" Name=\"type\" format=\"ascii\" RangeMin=\"0\" RangeMax=\"8\">\n";
    f << section([&](std::ostringstream& os, long long i) { os << (int)type[i] << " "; });
    f << "    </DataArray>\n";
    f << "    <DataArray type=\"Float64\" Name=\"v\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    f << section([&](std::ostringstream& os, long long i) {
        os << v[3 * i] << " " << v[3 * i + 1] << " " << v[3 * i + 2] << " ";
    });
    f << "    </DataArray>\n";
    f << "    <DataArray type=\"Float64\" Name=\"pressure\" format=\"ascii\" RangeMin=\"0\" RangeMax=\"2\">\n";
    f << section([&](std::ostringstream& os, long long i) { os << pr[i] << " "; });
    f << "    </DataArray>\n";
    if (vis) {
        f << "    <DataArray type=\"Float64\" Name=\"dynVisc\" format=\"ascii\" RangeMin=\"0\" RangeMax=\"2\">\n";
        f << section([&](std::ostringstream& os, long long i) { os << vi[i] << " "; });
        f << "    </DataArray>\n";
    }
    if (fs) {
        f << "    <DataArray type=\"Float64\" Name=\"AAAmass\" format=\"ascii\" RangeMin=\"0\" RangeMax=\"2\">\n";
        f << section([&](std::ostringstream& os, long long i) { os << ms[i] << " "; });
        f << "    </DataArray>\n";
    }
    if (dem) {
        f << "    <DataArray type=\"Int16\" Name=\"solidIndex\" format=\"ascii\" RangeMin=\"0\" RangeMax=\"8\">\n";
        f << section([&](std::ostringstream& os, long long i) { os << so[i] << " "; });
        f << "    </DataArray>\n";
    }
    f << "   </PointData>\n";
    f << "   <CellData>\n";
    f << "   </CellData>\n";
    f << "  </Piece>\n";
    f << " </ImageData>\n";
    f << "</VTKFile>\n";
    if (!f) return seterr(HB_ERR_ARG, "write failed: %s", path);
    return HB_OK;
}

int hb_profile_phases(hb_ctx* c, int32_t nsteps, double* us, int32_t* nphases) {
    if (!c || !c->initialized || !us || !nphases) return seterr(HB_ERR_ARG, "null argument or not initialised");
    if (!(c->P.dem_solve && c->d.E > 0)) { *nphases = 0; return HB_OK; }
    const int np = 2 + 2 * c->d.multi;  // barrier stamps of the cooperative kernel
    unsigned long long* ts = nullptr;
    int rc = dalloc(&ts, (size_t)np * nsteps);
    if (rc) return rc;
    CK(cudaMemset(ts, 0, sizeof(unsigned long long) * np * nsteps));
    std::vector<cudaEvent_t> ev(4 * (size_t)nsteps);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    for (int s = 0; s < nsteps; ++s) {
        if (launch_cycle_coop(c, 1, 1, 1, ts + (size_t)s * np)) { cudaFree(ts); return seterr(HB_ERR_CUDA, "cycle launch failed"); }
        launch_couple(c, false, c->cur, ev.data() + 4 * (size_t)s);
        if (c->P.free_surface) launch_fs_step(c, c->cur);
        launch_lb_step(c, c->cur);
        if (c->has_dynwall) launch_lb_wallforce(c, c->cur);
        c->cur ^= 1;
        c->reduce_pending = sums_lag(c);  // the sums lag the lattice step
        ++c->steps;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (c->mode_val != 1) c->mirror_valid = !c->P.lb_solve;
    std::vector<unsigned long long> h((size_t)np * nsteps);
    CK(cudaMemcpy(h.data(), ts, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost));
    cudaFree(ts);
    const int nint = np - 1;  // intervals between the recorded barriers
    for (int k = 0; k < nint; ++k) {
        double acc = 0.0;
        for (int s = 0; s < nsteps; ++s) acc += (double)(h[(size_t)s * np + k + 1] - h[(size_t)s * np + k]) * 1e-3;
        us[k] = acc / nsteps;
    }
    for (int k = 0; k < 3; ++k) {  // coupling: list reset, mask pass (pop + claim), commit
        double acc = 0.0;
        for (int s = 0; s < nsteps; ++s) {
            float m = 0.f;
            CK(cudaEventElapsedTime(&m, ev[4 * (size_t)s + k], ev[4 * (size_t)s + k + 1]));
            acc += m * 1e3;
        }
        us[nint + k] = acc / nsteps;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *nphases = nint + 3;
    return HB_OK;
}

int hb_time_cycles(hb_ctx* c, int32_t nsteps, float* ms_total, float* ms_lb_kernel, int32_t* kernels_per_cycle) {
    if (!c || !c->initialized) return seterr(HB_ERR_STATE, "not initialised");
    if (nsteps <= 0) return seterr(HB_ERR_ARG, "nsteps <= 0");
    CK(cudaStreamSynchronize(c->stream));
    // whole cycles replayed from the graphs
    CK(cudaMemsetAsync(c->mode, 0, sizeof(int), c->stream));
    c->mode_val = 0;
    c->mirror_valid = !c->P.lb_solve;
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s < nsteps; ++s) {
        CK(cudaGraphLaunch(c->gexec[c->cur], c->stream));
        c->force_dirty = false;
        if (c->P.lb_solve) { c->cur ^= 1; c->reduce_pending = sums_lag(c); }
        ++c->steps;
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    if (ms_total) *ms_total = ms;
    if (kernels_per_cycle) *kernels_per_cycle = c->kernels_per_cycle;
    // the collide+stream kernel alone, bracketed by events on its own stream inside the
    // same cycles launched kernel by kernel
    if (ms_lb_kernel && c->P.lb_solve) {
        std::vector<cudaEvent_t> ev(2 * nsteps);
        for (auto& e : ev) CK(cudaEventCreate(&e));
        const bool dem = c->P.dem_solve && c->d.E > 0;
        for (int s = 0; s < nsteps; ++s) {
            if (dem && launch_cycle_coop(c, 1, 1, 1)) return seterr(HB_ERR_CUDA, "cycle launch failed");
            if (dem) launch_couple(c, false, c->cur);
            if (c->P.free_surface) launch_fs_step(c, c->cur);
            CK(cudaEventRecord(ev[2 * s], c->stream));
            launch_lb_step(c, c->cur);
            CK(cudaEventRecord(ev[2 * s + 1], c->stream));
            if (c->has_dynwall) launch_lb_wallforce(c, c->cur);
            c->cur ^= 1;
            c->reduce_pending = sums_lag(c);  // the sums lag the lattice step
            ++c->steps;
        }
        CK(cudaStreamSynchronize(c->stream));
        double tot = 0.0;
        for (int s = 0; s < nsteps; ++s) {
            float m = 0.f;
            CK(cudaEventElapsedTime(&m, ev[2 * s], ev[2 * s + 1]));
            tot += m;
        }
        *ms_lb_kernel = (float)(tot / nsteps);
        for (auto& e : ev) cudaEventDestroy(e);
    }
    CK(cudaGetLastError());
    return HB_OK;
}

// ---- reverse (adjoint) ---------------------------------------------------------------

int hb_adjoint_forward(hb_ctx* c, const hb_adjoint_cfg* cfg, double* J) {
    if (!c) return seterr(HB_ERR_ARG, "ctx is NULL");
    std::string e;
    const int rc = hb::adjoint_run(c, cfg, false, J, nullptr, nullptr, nullptr, e);
    return rc ? seterr(rc, "%s", e.c_str()) : HB_OK;
}

int hb_adjoint_drag(hb_ctx* c, const hb_adjoint_cfg* cfg, double* J, double* dJ_dF, double* dJ_dtau,
                    double* dJ_dUin) {
    if (!c) return seterr(HB_ERR_ARG, "ctx is NULL");
    std::string e;
    const int rc = hb::adjoint_run(c, cfg, true, J, dJ_dF, dJ_dtau, dJ_dUin, e);
    return rc ? seterr(rc, "%s", e.c_str()) : HB_OK;
}

int hb_adjoint_timing(hb_ctx* c, float* ms_forward, float* ms_reverse, int64_t* forward_steps,
                      int64_t* reverse_steps) {
    if (!c) return seterr(HB_ERR_ARG, "ctx is NULL");
    if (hb::adjoint_timing(c, ms_forward, ms_reverse, forward_steps, reverse_steps))
        return seterr(HB_ERR_STATE, "no adjoint call has run on this context");
    return HB_OK;
}

}  // extern "C"
