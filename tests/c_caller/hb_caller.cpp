// Test infrastructure: a C++11 host driver of the library's C-ABI, written the way the
// reference's own driver (hybird.cpp:245-344, goCycle hybird.cpp:35-66) would call it
// after parseConfigFile (hybird.cpp:132-223) has filled hb_params: create -> init ->
// cycles -> synchronize -> downloads -> destroy, every status checked.
//
// Usage: hb_caller <precision 0|1|2> <cycles>
// Prints the element state and a checksum of the lattice as text lines with %.17g values.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hybird_gpu.h"

namespace {

int check(int rc, const char* what) {
    if (rc != HB_OK) {
        std::fprintf(stderr, "%s failed: %d (%s)\n", what, rc, hb_last_error());
        std::exit(2);
    }
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    const int precision = argc > 1 ? std::atoi(argv[1]) : HB_FP64;
    const int cycles = argc > 2 ? std::atoi(argv[2]) : 20;

    // the cfg keys of a small coupled box: 16^3 lattice, no-slip walls, gravity along -z,
    // two spheres (lattice units, LB.cpp:85-188, DEM.cpp:13-183)
    hb_params p;
    std::memset(&p, 0, sizeof(p));
    p.lb_size[0] = p.lb_size[1] = p.lb_size[2] = 16;
    for (int k = 0; k < 6; ++k) p.boundary[k] = HB_T_STATWALL;
    p.units[0] = p.units[1] = p.units[2] = 1.0;
    p.init_visc = 0.1;
    p.lbF[2] = -1e-4;
    p.force_field = 1;
    p.collision = HB_BGK;
    p.trt_magic = 3.0 / 16.0;
    p.precision = precision;
    p.lb_solve = 1;
    p.dem_solve = 1;
    p.multi_step = 3;
    p.contact_model = HB_LINEAR;
    p.density = 2.5;
    p.linear_stiff = 1e3;
    p.young_mod = 1.0;
    p.poisson = 0.3;
    p.restitution = 0.8;
    p.visc_tang = 0.5;
    p.friction_part = 0.5;
    p.friction_wall = 0.5;

    const double radius[2] = {2.5, 2.2};
    const double x0[6] = {6.3, 10.2, 7.1, 9.4, 6.6, 9.9};  // component-major: x, x, y, y, z, z
    const double zero[6] = {0, 0, 0, 0, 0, 0};
    hb_elements el;
    el.count = 2;
    el.radius = radius;
    el.x0 = x0;
    el.x1 = zero;
    el.w0 = zero;
    el.q0 = nullptr;
    el.size = nullptr;

    hb_ctx* ctx = nullptr;
    check(hb_create(&p, &ctx), "hb_create");
    check(hb_init(ctx, &el, nullptr), "hb_init");
    check(hb_cycle(ctx, cycles), "hb_cycle");
    check(hb_synchronize(ctx), "hb_synchronize");

    const size_t N = 16 * 16 * 16;
    std::vector<uint8_t> type(N), inside(N);
    std::vector<double> f(19 * N), n(N), u(3 * N);
    check(hb_download_lattice(ctx, type.data(), inside.data(), nullptr, f.data(), n.data(), u.data(), nullptr,
                              nullptr, nullptr),
          "hb_download_lattice");
    std::vector<double> ex0(6), ex1(6), fh(6), mh(6);
    check(hb_download_elements(ctx, ex0.data(), ex1.data(), nullptr, nullptr, fh.data(), mh.data(), nullptr,
                               nullptr, nullptr, nullptr, nullptr),
          "hb_download_elements");
    hb_status st;
    check(hb_get_status(ctx, &st), "hb_get_status");
    check(hb_destroy(ctx), "hb_destroy");

    double fsum = 0.0, usum = 0.0;
    long active = 0, in = 0;
    for (size_t i = 0; i < N; ++i) {
        if (type[i] != HB_T_FLUID && type[i] != HB_T_INTERFACE) continue;
        ++active;
        in += inside[i];
        for (int j = 0; j < 19; ++j) fsum += f[j * N + i];
        usum += std::fabs(u[i]) + std::fabs(u[N + i]) + std::fabs(u[2 * N + i]);
    }
    std::printf("active %ld inside %ld status_active %lld numeric %d\n", active, in, (long long)st.active_nodes,
                st.numeric_error);
    std::printf("fsum %.17g usum %.17g\n", fsum, usum);
    const char* names[4] = {"x0", "x1", "FHydro", "MHydro"};
    const std::vector<double>* arrs[4] = {&ex0, &ex1, &fh, &mh};
    for (int k = 0; k < 4; ++k) {
        std::printf("%s", names[k]);
        for (double v : *arrs[k]) std::printf(" %.17g", v);
        std::printf("\n");
    }
    return 0;
}
