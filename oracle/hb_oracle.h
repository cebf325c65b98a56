/*
 * hb_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++/OpenMP FP64 restatement of hybird's time-step path (LB stream+collide,
 * free surface, LB-DEM coupling, DEM), written from the reference's algorithm and
 * following its arithmetic order so that it reproduces the reference bit-for-bit on
 * the fixtures in tests/golden/ (generated from the reference itself).  It is the
 * checker for the CUDA library and the timed CPU baseline; the product never links it.
 */
#ifndef HB_ORACLE_H
#define HB_ORACLE_H

#include "../include/hybird_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hbo_sim hbo_sim;

/* init as LB::latticeBolzmannInit + DEM::discreteElementInit; NULL on error */
hbo_sim* hbo_create(const hb_params* p, const hb_elements* e, const hb_objects* o);
/* the same with cylinders (curved walls, LB.cpp:552-603) */
hbo_sim* hbo_create_cyl(const hb_params* p, const hb_elements* e, const hb_objects* o, const hb_cylinders* cy);
void hbo_destroy(hbo_sim* s);
const char* hbo_last_error(void);
/* nsteps goCycle()s (hybird.cpp:35-66) */
int hbo_cycle(hbo_sim* s, int nsteps);
/* individual phases, same semantics as the reference methods */
int hbo_dem_step(hbo_sim* s);
int hbo_fs_step(hbo_sim* s);
int hbo_coupling_step(hbo_sim* s);
int hbo_lb_step(hbo_sim* s);
int hbo_set_threads(int n);

int64_t hbo_nodes(const hbo_sim* s);
int64_t hbo_active(const hbo_sim* s);
int hbo_get_lattice(const hbo_sim* s, uint8_t* type, uint8_t* inside, uint32_t* solid,
                    uint8_t* has_node, double* f, double* n, double* u, double* mass,
                    double* visc, double* hydro_force);
int hbo_set_lattice(hbo_sim* s, const double* f, const double* n, const double* u,
                    const double* mass, const double* visc);
int hbo_set_body_force(hbo_sim* s, const double* force);
int hbo_get_elements(const hbo_sim* s, double* x0, double* x1, double* w, double* q0,
                     double* fhydro, double* mhydro, double* fparticle, double* fwall,
                     double* mparticle, double* mwall, double* fluid_volume);
/* raw neighborTable (pairs in reference order), returns the pair count */
int64_t hbo_get_pairs(const hbo_sim* s, uint32_t* pairs, int64_t capacity);
int64_t hbo_get_interface(const hbo_sim* s, uint32_t* cells, int64_t capacity);
int hbo_get_walls(const hbo_sim* s, double* fhydro, double* fparticle, int32_t* nwalls);
/* objects[].FParticle of the last substep (DEM.cpp:2103, 2132) [3*nobjects] */
int hbo_get_objects(const hbo_sim* s, double* fparticle, int32_t* nobjects);
double hbo_total_mass(const hbo_sim* s);
int hbo_dem_scalars(const hbo_sim* s, double* out /* demTime,maxDisp,nebrRange,deltat */);
/* drag on the objects along axis from the last step's post-collision populations */
double hbo_object_drag(const hbo_sim* s, int axis);

#ifdef __cplusplus
}
#endif
#endif
