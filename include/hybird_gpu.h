/*
 * hybird_gpu.h -- C-ABI of the GB300 (sm_103a) time-step library for hybird.
 *
 * One opaque context owns every device buffer of one simulation on one GPU.  The
 * reference's per-step class methods (LB::latticeBolzmannStep, LB.h:159; LB::
 * latticeBoltzmannFreeSurfaceStep, LB.h:161; LB::latticeBoltzmannCouplingStep, LB.h:160;
 * DEM::discreteElementStep, DEM.h:137) become one-line forwarders into these calls;
 * every call returns an int status (HB_OK == 0) instead of calling exit() as the
 * reference does (macros.h:8, LB.cpp:1057, LB.cpp:1460).
 *
 * Units: every quantity crossing this boundary is in the reference's lattice units
 * with unitLength = unitTime = unitDensity = 1 (LB.cpp:93-98); hb_create rejects other
 * unit values.  Lattice arrays are indexed like the reference, i = x + y*X + z*X*Y
 * (LB.cpp:2314-2370); per-direction and per-component arrays are structure-of-arrays,
 * component-major: f[j*N + i], u[c*N + i].
 */
#ifndef HYBIRD_GPU_H
#define HYBIRD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define HB_OK               0
#define HB_ERR_ARG          1   /* bad argument, NULL pointer, size mismatch          */
#define HB_ERR_UNSUPPORTED  2   /* feature outside the implemented path               */
#define HB_ERR_CUDA         3   /* CUDA runtime error (message via hb_last_error)      */
#define HB_ERR_NOMEM        4   /* device allocation failed                            */
#define HB_ERR_CAPACITY     5   /* a fixed-capacity device list overflowed             */
#define HB_ERR_STATE        6   /* call out of order (e.g. step before upload)         */
#define HB_ERR_NUMERIC      7   /* NaN/Inf detected in density or velocity             */

/* ---- enumerations ------------------------------------------------------------------ */
#define HB_FP64   0   /* populations stored and computed in FP64                           */
#define HB_FP32   1   /* populations stored as f_i - w_i*rho0 in FP32, FP32 compute        */
#define HB_FP16S  2   /* populations stored as scaled FP16 deviations, FP32 compute        */

#define HB_BGK    0   /* single relaxation time, node.cpp:158-165                          */
#define HB_TRT    1   /* two relaxation times (magic parameter), not in the reference      */

#define HB_DIRECT_FORCING 0 /* the reference's coupling: -eps (u - u_p) on nodes inside
                                particles, which stay fluid (LB.cpp:1851-1919)               */
#define HB_MOVING_BB      1 /* not in the reference (its branch is commented out, LB.cpp:
                                1247-1276): nodes inside particles are solid and fluid links
                                into them bounce back with the particle's local velocity     */

#define HB_LINEAR   0 /* ContactModel LINEAR  (elmt.h:137)                                 */
#define HB_HERTZIAN 1 /* ContactModel HERTZIAN (elmt.h:137)                                */

/* node type codes, identical to nodeType::t (node.h:75-86) */
#define HB_T_FLUID     0
#define HB_T_GAS       2
#define HB_T_INTERFACE 3
#define HB_T_PERIODIC  4
#define HB_T_SLIPSTAT  5
#define HB_T_SLIPDYN   6
#define HB_T_STATWALL  7
#define HB_T_DYNWALL   8
#define HB_T_CURVED    9

/* ---- parameters -------------------------------------------------------------------- */
/* Mirrors the cfg keys parsed by LB::latticeBoltzmannGet (LB.cpp:85-188),
 * DEM::discreteElementGet (DEM.cpp:13-183) and parseConfigFile (hybird.cpp:132-223). */
typedef struct hb_params {
    int32_t lb_size[3];        /* lbSizeX/Y/Z: nodes incl. the two boundary layers          */
    int32_t boundary[6];       /* boundary0..5 (x-,x+,y-,y+,z-,z+): 4, 5, 6, 7 or 8         */
    double  units[3];          /* unitLength, unitTime, unitDensity: must be 1.0            */
    double  init_visc;         /* initVisc (kinematic, lattice units): tau = 0.5 + 3 nu     */
    double  init_velocity[3];  /* initVelocityX/Y/Z                                          */
    double  lbF[3];            /* lbFX/Y/Z body force (also DEM gravity, DEM.cpp:194)        */
    int32_t force_field;       /* forceFieldSolve: 0 zeroes lbF in collision (LB.cpp:1074)   */
    int32_t non_newtonian;     /* nonNewtonianSolve (Bingham)                                */
    double  plastic_visc;      /* plasticVisc                                                */
    double  yield_stress;      /* yieldStress                                                */
    int32_t turbulence;        /* turbulenceSolve (Smagorinsky)                              */
    double  turb_const;        /* turbConst = Cs^2                                           */
    int32_t free_surface;      /* freeSurfaceSolve                                           */
    int32_t collision;         /* HB_BGK | HB_TRT                                            */
    double  trt_magic;         /* TRT magic parameter Lambda (e.g. 3/16)                     */
    int32_t precision;         /* HB_FP64 | HB_FP32 | HB_FP16S                               */
    double  gas_box[2];        /* dam-break column: gas where x >= gx*X or z >= gz*Z;
                                  {0,0} disables (interface init as LB.cpp:787-814)          */
    int32_t lb_solve;          /* lbSolve: 0 runs DEM only (hybird.cpp:49-64)                */
    /* DEM (DEM.cpp:13-183) */
    int32_t dem_solve;         /* demSolve                                                   */
    int32_t multi_step;        /* multiStep (>= 1): DEM substeps per LB step                 */
    int32_t contact_model;     /* HB_LINEAR | HB_HERTZIAN                                    */
    double  density;           /* particle density                                           */
    double  linear_stiff;      /* linearStiff                                                */
    double  young_mod;         /* youngMod  (HERTZIAN)                                       */
    double  poisson;           /* poisson   (HERTZIAN)                                       */
    double  restitution;       /* restitution                                                */
    double  visc_tang;         /* viscTang                                                   */
    double  friction_part;     /* frictionCoefPart                                           */
    double  friction_wall;     /* frictionCoefWall                                           */
    double  num_visc;          /* numVisc                                                    */
    /* capacities of the fixed-size device lists (0 = library default); the reference's
       lists are unbounded (DEM.cpp:1369-1494, LB.cpp:1592-1618): an overflow here stops
       nothing on the device but makes hb_synchronize return HB_ERR_CAPACITY naming the list */
    int64_t cap_neighbors;     /* DEM candidate partners kept per particle (default 48)      */
    int64_t cap_interface;     /* free-surface interface cells listed per step (default: all nodes) */
    double  slip_coefficient;  /* slipCoefficient S of the slip walls 5/6 (LB.cpp:1154-1155) */
    /* HB_DIRECT_FORCING (default, the reference's scheme) | HB_MOVING_BB.  Moving
       bounce-back: a fluid node i with link j onto a node l inside particle p takes
       f_i[opp j] = fs_i[j] - BBi, BBi = 6 n_i w_j (u_l . c_j), u_l = V_e + omega_e x
       (x_l - X_e) of p's element e; the element gains (2 (fs_i[j] - w_j) - BBi) c_j and its
       moment about X_e (node::bounceBackForce, node.cpp:283-291).  A node the particle
       uncovers is refilled with f_eq(rho, u_l), rho the mean density of its fluid links (1
       without any); a node it covers drops its populations.  Single spheres without
       periodic faces, no free surface, no cylinders (HB_ERR_UNSUPPORTED otherwise). */
    int32_t coupling;
} hb_params;

/* Elements (DEM.cpp:81-127 particle file row): single spheres, or 2-4 spheres when size is given. */
typedef struct hb_elements {
    int32_t count;
    const double* radius;      /* [count]                                                    */
    const double* x0;          /* [3*count] centre, component-major                          */
    const double* x1;          /* [3*count] velocity                                         */
    const double* w0;          /* [3*count] angular velocity                                 */
    const double* q0;          /* [4*count] orientation quaternion (p,q,r,s); NULL = (1,0,0,0) */
    const int32_t* size;       /* [count] spheres of the element, 1..4, at the prototype
                                  positions of DEM::compositeProperties (DEM.cpp:404-433);
                                  NULL = single spheres                                       */
} hb_elements;

/* Fixed spherical objects (DEM.cpp:129-173 object file row); they become static-wall
 * lattice nodes (LB.cpp:535-550) and DEM contact partners (DEM.cpp:2060-2136). */
typedef struct hb_objects {
    int32_t count;
    const double* radius;      /* [count]   */
    const double* x0;          /* [3*count] */
    const double* x1;          /* [3*count] velocity (contact only) */
} hb_objects;

/* Device-side status word, read back at output steps (all counters since the last read). */
typedef struct hb_status {
    int32_t numeric_error;     /* NaN/Inf seen in rho or u                                   */
    int32_t capacity_error;    /* a device list overflowed                                   */
    int32_t unsupported_link;  /* an active node linked to an unsupported node type (the
                                  reference's TYPE ERROR exit, LB.cpp:1458-1461)            */
    int32_t reserved;
    int64_t interface_cells;   /* current interface count                                    */
    int64_t active_nodes;      /* fluid + interface nodes (activeNodes.size())               */
    int64_t pairs;             /* DEM candidate pairs (neighborTable.size()/2)               */
    int64_t contacts;          /* overlapping pairs in the last DEM substep                  */
    double  mass_surplus;      /* FP64 free-surface ledger of the last step                  */
    double  total_mass;        /* FP64 sum of mass over active non-particle nodes            */
} hb_status;

/* Output-step quantities of the reference's export.dat line (IO::outputStep,
 * IO.cpp:132-198) and of DEM::updateEnergy (DEM.cpp:2226-2276), in lattice units. */
typedef struct hb_export {
    double  max_fluid_speed;      /* sqrt(max |u|^2) over active nodes (IO.cpp:835-851)         */
    double  total_fluid_mass;     /* sum of mass over active nodes outside particles (IO.cpp:987-999) */
    double  plastic_percent;      /* 100 * plastic / active (IO.cpp:969-985)                     */
    int64_t active_nodes;         /* fluid + interface nodes                                     */
    int64_t plastic_nodes;        /* active nodes with visc > 0.95 (1.8 - 0.5) / 3               */
    double  max_particle_speed;   /* sqrt(max |x1|^2) over elements (IO.cpp:853-862)             */
    double  max_particle_spin;    /* sqrt(max |wGlobal|^2) (IO.cpp:864-871)                      */
    double  collision_force;      /* sum |FParticle| + |FWall| in element order (IO.cpp:1074-1084) */
    double  hydraulic_force;      /* sum |FHydro| in element order (IO.cpp:1064-1072)            */
    double  particle_mass;        /* sum of element masses (IO.cpp:1001-1010)                    */
    double  object_force[3];      /* sum of objects' FParticle (IO.cpp:1097-1106)                */
    double  energy_kin, energy_rot_kin, energy_tr_kin, energy_grav, energy_total;
} hb_export;

/* Cylinders (the reference's cylinder class, utils.h:85-110; problem code creates them,
 * DEM.cpp:871-935): every lattice node outside a cylinder becomes a curved wall (9) with
 * Mei-Luo-Shyy interpolated bounce-back (LB.cpp:552-603, 1278-1319). */
typedef struct hb_cylinders {
    int32_t count;
    const double* p1;          /* [3*count] axis point 1                                     */
    const double* p2;          /* [3*count] axis point 2                                     */
    const double* radius;      /* [count]                                                    */
    const double* omega;       /* [3*count] angular velocity (used when moving)              */
    const int32_t* moving;     /* [count] 1: rotating (curved-node velocity omega x r)       */
} hb_cylinders;

typedef struct hb_ctx hb_ctx;

/* ---- lifecycle ------------------------------------------------------------------- */
/* Cylinders for the next hb_init (call between hb_create and hb_init): curved walls for
 * the lattice and contact partners of the particles (DEM.cpp:1535-1550, 1719-2058; at most
 * 4 with moving particles).  Not combined with a free surface: hb_init returns
 * HB_ERR_UNSUPPORTED. */
int hb_set_cylinders(hb_ctx* ctx, const hb_cylinders* cylinders);
/* Replaces the LB/DEM constructors + LB::latticeDefinition (LB.cpp:42-83) and
 * DEM::discreteElementInit parameter setup (DEM.cpp:185-297).  Allocates all device
 * memory once; nothing is allocated per step. */
int hb_create(const hb_params* params, hb_ctx** out);
int hb_destroy(hb_ctx* ctx);
const char* hb_last_error(void);

/* Builds the initial state on the device, as LB::latticeBolzmannInit does
 * (LB.cpp:190-219): lattice boundaries, walls (DEM.cpp:435-633), particle flags
 * (LB.cpp:475-495), objects (LB.cpp:535-550), interface (LB.cpp:787-814), hydrostatic
 * variables (LB.cpp:909-944), wall nodes (LB.cpp:946-996) and f = f_eq.
 * elements/objects may be NULL. */
int hb_init(hb_ctx* ctx, const hb_elements* elements, const hb_objects* objects);

/* Overwrites the lattice state with a host-built one (the reference's own init, or a
 * checkpoint).  N = X*Y*Z.  type[N] node codes, inside[N] particle flags, solid[N]
 * solid indices, f[19*N] (NULL: f = f_eq(n,u) as node::initialize, node.cpp:26-61),
 * n[N], u[3*N], mass[N], visc[N] (NULL: init_visc). */
int hb_upload_lattice(hb_ctx* ctx, const uint8_t* type, const uint8_t* inside,
                      const uint32_t* solid, const double* f, const double* n,
                      const double* u, const double* mass, const double* visc);

/* ---- time step (goCycle order, hybird.cpp:35-66) ----------------------------------- */
int hb_dem_step(hb_ctx* ctx);        /* DEM::discreteElementStep        DEM.cpp:331-376  */
int hb_fs_step(hb_ctx* ctx);         /* LB::latticeBoltzmannFreeSurfaceStep LB.cpp:235-245 */
int hb_coupling_step(hb_ctx* ctx);   /* LB::latticeBoltzmannCouplingStep LB.cpp:247-280  */
int hb_lb_step(hb_ctx* ctx);         /* LB::latticeBolzmannStep         LB.cpp:221-233  */
/* nsteps whole cycles (DEM, free surface, coupling, LB) replayed from one CUDA graph.  The
 * last cycle of the call also writes every node's density, velocity and hydrodynamic force
 * (the reference's node fields, which hb_download_lattice, hb_export_values and the VTK
 * writer read) unless the lattice mirror is off. */
int hb_cycle(hb_ctx* ctx, int32_t nsteps);
/* on (default, 1): hb_cycle's last cycle writes the node fields as above; off (0): the
 * cycles write them only where a later phase of the step reads them (the state itself is
 * the same), for a driver that reads element state only.  While the last cycles ran with
 * the mirror off (or through hb_time_cycles / hb_profile_phases), the entry points that
 * read those node fields return HB_ERR_STATE and hb_get_status leaves active_nodes and
 * total_mass at 0. */
int hb_set_lattice_mirror(hb_ctx* ctx, int32_t on);
/* The context's parameters (as last set: lbF follows hb_set_body_force) and its element
 * and object counts; any pointer may be NULL. */
int hb_get_params(hb_ctx* ctx, hb_params* out, int32_t* elements, int32_t* objects);
/* Changes the body force lbF used by the collision from the next step on (the reference
 * reads lb.lbF every collision, LB.cpp:1098-1111; problem code may change it).  With
 * particles the new value travels in the parameters of the cycle graphs' mask kernel,
 * which writes it before the lattice step: no launch of its own between two cycles. */
int hb_set_body_force(hb_ctx* ctx, const double* force /* [3] */);
int hb_synchronize(hb_ctx* ctx);

/* ---- download (output steps and tests) --------------------------------------------- */
/* Any pointer may be NULL.  f is the post-streaming population (the reference's
 * node::f between steps); n,u are the values of the last reconstruction (with u
 * shifted by half the force, as the reference leaves them after collision). */
int hb_download_lattice(hb_ctx* ctx, uint8_t* type, uint8_t* inside, uint32_t* solid,
                        double* f, double* n, double* u, double* mass, double* visc,
                        double* hydro_force);
/* Element state (component-major [3*count]); FHydro/MHydro as last computed by the
 * coupling (LB.cpp:1851-1919), FParticle/FWall/MParticle/MWall of the last substep. */
int hb_download_elements(hb_ctx* ctx, double* x0, double* x1, double* w, double* q0,
                         double* fhydro, double* mhydro, double* fparticle, double* fwall,
                         double* mparticle, double* mwall, double* fluid_volume);
/* The same download queued on the context stream behind the steps already issued; it
 * returns without waiting.  The arrays hold the values once hb_synchronize returns and
 * must stay valid until then.  Arrays registered with hb_host_register (page-locked and
 * mapped) are written by the gather kernel itself, so a driver can issue step after step
 * and read the element state of each without a copy or a stall; other arrays are filled
 * by copies on the stream (pageable memory takes the CUDA runtime's synchronous path). */
int hb_download_elements_async(hb_ctx* ctx, double* x0, double* x1, double* w, double* q0,
                               double* fhydro, double* mhydro, double* fparticle, double* fwall,
                               double* mparticle, double* mwall, double* fluid_volume);
/* Page-locks and maps (cudaHostRegister, mapped) / releases host memory the caller passes
 * to the asynchronous downloads and the element sink. */
int hb_host_register(void* p, size_t bytes);
int hb_host_unregister(void* p);
/* Element sink: the arrays (same fields and layout as hb_download_elements, each
 * registered with hb_host_register, any of them null) are written at the end of every
 * cycle hb_cycle runs, by a gather kernel inside the cycle graph -- a host driver that
 * reads the element state after every step (the reference's DEM::particles feeding its
 * output and its own loop, hybird.cpp:35-66) gets it with no launch or copy of its own.
 * After hb_synchronize the arrays hold the state after the last cycle.  All arrays null
 * removes the sink.  The call re-captures the cycle graphs (it synchronises the stream);
 * the arrays must stay registered and valid until the sink is removed or the context
 * destroyed. */
int hb_set_element_sink(hb_ctx* ctx, double* x0, double* x1, double* w, double* q0, double* fhydro,
                        double* mhydro, double* fparticle, double* fwall, double* mparticle,
                        double* mwall, double* fluid_volume);
/* Candidate pair list as sorted (min,max) pairs, like DEM::neighborTable
 * (DEM.cpp:1369-1494) after normalisation.  *count receives the pair count.  With
 * periodic faces a ghost particle is numbered E + g (g its index in hb_download_ghosts),
 * as in the reference's particles list; pairs of two ghosts (which carry no force) are
 * not kept. */
int hb_download_pairs(hb_ctx* ctx, uint32_t* pairs, int64_t capacity, int64_t* count);
/* Ghost particles of the last neighbour rebuild with periodic faces, like DEM::ghosts
 * (DEM.cpp:1586-1664): element index and shift (x, y, z per ghost).  *count receives
 * the ghost count; either array may be null. */
int hb_download_ghosts(hb_ctx* ctx, uint32_t* origin, double* shift, int64_t capacity, int64_t* count);
/* Interface cells, ascending node index.  *count receives the count. */
int hb_download_interface(hb_ctx* ctx, uint32_t* cells, int64_t capacity, int64_t* count);
/* Per-wall hydrodynamic force (walls[].FHydro, LB.cpp:1334) and particle force
 * (walls[].FParticle of the last substep, DEM.cpp:1123-1125, 1946, 1977) [3*nwalls];
 * *nwalls = count.  Either array may be NULL. */
int hb_download_walls(hb_ctx* ctx, double* fhydro, double* fparticle, int32_t* nwalls);
/* ---- checkpoint / restart ---------------------------------------------------------- */
/* No counterpart in the reference (its .restart file, DEM.cpp:2337-2420, is DEM metadata
 * and its recycle file six-digit particle rows).  Saves every device buffer that carries
 * state between steps plus the host step state; a context loaded from the file continues
 * bit-identically to the one that saved it.  The file is specific to this library
 * version and to the host's byte order. */
int hb_checkpoint_save(hb_ctx* ctx, const char* path);
/* Builds a new context (hb_create + hb_init from the saved parameters, particles and
 * objects) and restores the saved state into it. */
int hb_checkpoint_load(const char* path, hb_ctx** out);
/* IO::exportRecycleParticles (IO.cpp:486-535): the particle-file rows (index size radius
 * x0 x1 w0 q0 q1) of the current elements, default stream formatting, readable as a
 * particle file (DEM.cpp:81-127). */
int hb_write_recycle_particles(hb_ctx* ctx, const char* path);

/* ---- output mirror (IO.cpp:132-198, 698-1104) ------------------------------------- */
/* The export.dat quantities of the current state, computed on the device: node sums in
 * a fixed order (deterministic, not the reference's sequential rounding), element sums
 * in element order (the reference's own).  Call after hb_cycle/hb_synchronize. */
int hb_export_values(hb_ctx* ctx, hb_export* out);
/* The per-node arrays of IO::exportParaviewFluidOld (IO.cpp:698-831) packed on the
 * device: type (1 for nodes inside a particle, else the type code), v [3*N] (x, y, z per
 * node), pressure 0.3333333 (n - 1), dynVisc, mass, solidIndex; zero for nodes that own
 * no node object (gas, periodic, walls no non-wall node links to).  Any pointer may be
 * NULL.  Node fields are those of the last full mirror (hb_cycle's last step). */
int hb_vtk_fluid_fields(hb_ctx* ctx, int8_t* type, double* v, double* pressure, double* dyn_visc,
                        double* mass, uint32_t* solid_index);
/* Writes the fluid image-data file of IO::exportParaviewFluidOld (same layout and default
 * stream formatting; dynVisc with nonNewtonianSolve, AAAmass with freeSurfaceSolve,
 * solidIndex with demSolve). */
int hb_write_vtk_fluid(hb_ctx* ctx, const char* path);
/* Per-object particle force (objects[].FParticle of the last substep, DEM.cpp:1127-1129,
 * 2103, 2132) [3*nobjects], summed in the reference's contact order; *nobjects = count. */
int hb_download_objects(hb_ctx* ctx, double* fparticle, int32_t* nobjects);
int hb_get_status(hb_ctx* ctx, hb_status* status);

/* ---- measurement ------------------------------------------------------------------- */
/* Runs nsteps cycles on the context's stream bracketed by CUDA events and returns the
 * elapsed device time of the whole cycles and of the stream-collide kernel alone. */
int hb_time_cycles(hb_ctx* ctx, int32_t nsteps, float* ms_total, float* ms_lb_kernel,
                   int32_t* kernels_per_cycle);
/* Runs nsteps cycles with device timestamps at the grid barriers of the DEM/coupling
 * kernel and returns the mean duration (microseconds) of each phase in order:
 * element-force reduction, then (forces, correct+predict) per DEM substep, then the
 * three coupling-mask passes.  us must hold 4 + 2*multiStep values. */
int hb_profile_phases(hb_ctx* ctx, int32_t nsteps, double* us, int32_t* nphases);

/* ---- reverse (adjoint) ------------------------------------------------------------- */
/* No counterpart in the reference (it has no derivative code).  Objective: J = total
 * drag on the context's objects (fixed spheres, which the lattice holds as static wall
 * nodes, LB.cpp:535-550) along drag_axis, measured in the last of `steps` single-phase
 * steps: the sum over fluid->object links of 2 (fs_j - w_j rho0) c_j, the reference's
 * node::bounceBackForce (node.cpp:283-291) with BBi = 0.  The run starts from the
 * context's current populations (not changed by the call) and uses, instead of the
 * context's values, the relaxation time tau (TRT magic parameter and collision kind from
 * hb_params), the uniform body force F and the inlet field: moving-wall nodes (code 8)
 * on the planes x = 0 and x = X-1 move with velocity (u_in[y + Y*z], 0, 0); other
 * moving walls keep their node velocity.  Single-phase lattices only: no free surface,
 * no Bingham/Smagorinsky viscosity, no DEM elements (HB_ERR_UNSUPPORTED otherwise).
 * The gradient is taken by a hand-written reverse kernel with checkpoints of the state
 * every checkpoint_every steps in device memory and recomputation of each segment. */
typedef struct hb_adjoint_cfg {
    int32_t steps;             /* T >= 1                                                    */
    int32_t checkpoint_every;  /* K >= 1                                                    */
    int32_t precision;         /* HB_FP32 or HB_FP64: storage and arithmetic of the run     */
    int32_t drag_axis;         /* 0, 1, 2                                                   */
    double  tau;               /* relaxation time (> 0.5)                                   */
    double  body_force[3];     /* lbF                                                       */
    const double* inlet_velocity; /* host [Y*Z], index y + Y*z, or NULL for zero            */
} hb_adjoint_cfg;
/* Forward only: J (used for finite differences). */
int hb_adjoint_forward(hb_ctx* ctx, const hb_adjoint_cfg* cfg, double* J);
/* J and its gradient: dJ_dF[3], dJ_dtau[1], dJ_dUin[Y*Z] (host; any may be NULL). */
int hb_adjoint_drag(hb_ctx* ctx, const hb_adjoint_cfg* cfg, double* J, double* dJ_dF,
                    double* dJ_dtau, double* dJ_dUin);
/* Device time of the last adjoint call: the first forward pass, and the reverse pass
 * (segment recomputation + reverse steps); step counts of each. */
int hb_adjoint_timing(hb_ctx* ctx, float* ms_forward, float* ms_reverse,
                      int64_t* forward_steps, int64_t* reverse_steps);

/* ---- allocation-free entry point ----------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory:
 * an application that reserves the device memory up front and gives this library a
 * fixed budget (its own pool allocator owns the rest), and host loops with a latency
 * bound that cannot take the device-wide synchronisation a cudaMalloc or cudaFree may
 * cause.  Computes the moving-wall momentum exchange of one
 * streamed state (the quantity hb_download_walls reports, LB.cpp:1321-1341) from caller
 * device buffers and allocates nothing: its scratch is a fixed 152 KiB device array
 * inside the library, kept by every GPU that loads it until the process exits.
 *   f          [19*N] FP64 populations after streaming, component-major
 *   type       [N] node type codes (0..9; flag bits above the code are ignored),
 *              solid [N] wall index of wall nodes
 *   rho, mass  [N]; u [3*N] (wall-node velocities are read from u)
 *   wall_force [3*6+1] device output: per wall (Fx,Fy,Fz) in wall order, then the
 *              extra mass; stream: cudaStream_t or NULL for the default stream.
 * The first call on a device resolves the scratch address for that device and keeps
 * it: make that first call before any stream capture, and make no call after a
 * cudaDeviceReset of that device in the same process (the reset unloads the scratch).
 * Calls that overlap on the GPU share the scratch and race; the caller serialises them.
 * Each call overwrites every partial it reads, so no result depends on an earlier call.
 * Lattices above HB_NOALLOC_MAX_NODES give HB_ERR_ARG. */
#define HB_NOALLOC_MAX_NODES (1LL << 28)
int hb_wall_force_noalloc(const double* f, const uint8_t* type, const uint32_t* solid,
                          const double* rho, const double* u, const double* mass,
                          const int32_t* lb_size, const int32_t* boundary,
                          double* wall_force, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HYBIRD_GPU_H */
