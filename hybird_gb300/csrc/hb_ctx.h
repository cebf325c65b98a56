// hb_ctx.h -- host-side context of one simulation (device pointers, sizes, graph).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "hb_common.cuh"

// doubles per element in hb_dem_dev::base: x, xp, w, wp (6 x 3 each), q, qp (6 x 4 each),
// wG, wL, wpG, wpL, FH, MH, FP, FW, MP, MW (3 each), fvol, m, I (3), rad
constexpr int DEM_FIELDS = 6 * 3 * 4 + 6 * 4 * 2 + 4 * 3 + 6 * 3 + 1 + 1 + 3 + 1;

struct hb_cyl_host {            // one cylinder as given to hb_set_cylinders
    double p1[3], p2[3], R, omega[3];
    int moving;
};

struct hb_dem_dev {             // element state, FP64, component-major [3E] / [4E]
    int E = 0;
    double* base = nullptr;     // one allocation holding every field below
    double *x[6], *xp[6], *w[6], *wp[6];
    double *q[6], *qp[6];
    double *wG, *wL, *wpG, *wpL;
    double *FH, *MH, *FP, *FW, *MP, *MW;
    double *fvol, *m, *I, *rad;
    double* alt = nullptr;      // [9E] second copy of the predicted position, velocity and global spin
    float* pf = nullptr;        // [12(E+gcap)] FP32 centre/velocity/wGlobal(+pad) per particle (ghosts after the elements)
    int* plain = nullptr;       // [E] 1: orientation stays the identity (component-parallel Gear)
    // neighbour structures
    int* cell_of = nullptr;     // [E + gcap]
    int* cell_cnt = nullptr;    // [nc]
    int* cell_start = nullptr;  // [nc+1]
    int* cell_fill = nullptr;   // [nc]
    int* cell_items = nullptr;  // [E + gcap]
    int* nbr = nullptr;         // [E*nbr_cap]
    double* npc = nullptr;      // [4*E*nbr_cap] per candidate pair (single spheres): effMass,
                                // effRad and the linear model's two damping coefficients
    int nbr_cap = hb::NBR_CAP;  // candidate partners kept per particle
    int* nbr_cnt = nullptr;     // [E]
    int* wall_of = nullptr;     // [E] first wall in range or -1
    int* obj = nullptr;         // [E*OBJ_CAP]
    int* obj_cnt = nullptr;     // [E]
    int* cyl_of = nullptr;      // [E] first cylinder in range or -1
    double* wrec = nullptr;     // [7E] last substep's wall contact per element: flag, normal, tangential force
    double* orec = nullptr;     // [7E*OBJ_CAP] the same per (element, object slot)
    double* react = nullptr;    // [3*(MAX_WALLS + O)] wall and object FParticle (ordered sums of the records)
    uint32_t* claim_list = nullptr;  // [2N] (node, particle) pairs joined by the coupling in this step
    int* claim_cnt = nullptr;
    unsigned int* mask_done = nullptr;  // finished blocks of the mask pass (its last block commits)
    uint32_t* pop_list = nullptr;    // [N] nodes a particle uncovered in this step (moving bounce-back)
    int* pop_cnt = nullptr;
    double* pop_rho = nullptr;       // [N] their refill density
    void* boxes = nullptr;      // [E+gcap] per-particle spheres of the current step (coupling masks)
    void* gargs = nullptr;      // device copy of the DEM/coupling parameter blocks
    double* scal = nullptr;     // device scalars: [0]=maxDisp [1]=rebuild flag [2]=contacts
    int* contacts = nullptr;    // overlapping pairs counter of the last substep
    double* partial = nullptr;  // per-block maxima for the displacement trigger
    unsigned int* done = nullptr;  // last-block counter
    int ncells = 0;
    int nCells[3] = {0, 0, 0};
    double cellWidth[3] = {0, 0, 0};
    double nebrRange = 0.0, trigger = 0.0;
    double dt = 1.0;
    int multi = 1;
    double dampCoeff = 0, knConst = 0, ksConst = 0;
    // periodic faces (DEM.cpp:937-989) and ghost particles (DEM.cpp:1554-1664)
    int npbc = 0;
    double pbc_p[3][3], pbc_v[3][3];
    int gcap = 0;               // ghost slots: 6 per particle (3 faces + 3 corners)
    int* gmeta = nullptr;       // [0] ghosts of the last rebuild, [1] 1: particle nodes need a re-mark
    int* gorig = nullptr;       // [gcap] particle each ghost copies
    double* gvec = nullptr;     // [3*gcap] its shift (component-major, stride gcap)
    int* comp = nullptr;        // [6P] ghost particle indices (P + g) of each particle, in creation order
    int* ccnt = nullptr;        // [P]
    int* ecomp = nullptr;       // [6P] ghosts of each element (from 6*efirst[e]), in creation order
    int* eccnt = nullptr;       // [E]
    double* px = nullptr;       // [3*(P+gcap)] particle centres, corrected (stride P+gcap)
    // particles (DEM.cpp:222-239): element e owns the P-index range efirst[e] .. efirst[e+1]-1,
    // one sphere per prototype position (DEM.cpp:404-433); ghosts follow as P + g
    int P = 0;                  // standard particles
    int gen = 0;                // 1: periodic faces or multi-sphere elements (per-particle path)
    int* pkey = nullptr;        // [P+gcap] element of every particle
    int* efirst = nullptr;      // [E+1]
    int* esize = nullptr;       // [E] spheres of the element (1..4)
    double* proto = nullptr;    // [3P] prototype position of each particle, radius units (component-major)
    double* ppos = nullptr;     // [3(P+gcap)] predicted centre of every particle in the substep
    double* pvel = nullptr;     // [3(P+gcap)] its velocity (element velocity + spin x radiusVec)
    double* prv = nullptr;      // [3(P+gcap)] radiusVec: centre - element centre
    double* pF = nullptr;       // [12P] per-particle FParticle, MParticle, FWall, MWall of the substep
    double* pcen = nullptr;     // [3(P+gcap)] corrected element centre (+ ghost shift) seen by the coupling
    uint32_t* remark = nullptr; // [N] last covering particle + 1 during a re-mark (LB.cpp:1826-1849)
    // objects
    int O = 0;
    int O_std = 0;              // objects as uploaded; the rest are periodic images (DEM.cpp:990-1063)
    double* obj_x0 = nullptr;   // [3*O]
    double* obj_x1 = nullptr;   // [3*O]
    double* obj_r = nullptr;    // [O]
    // walls (boundary planes, DEM.cpp:435-633)
    int nw = 0;
    double wall_p[hb::MAX_WALLS][3], wall_n[hb::MAX_WALLS][3];
    int wall_code[hb::MAX_WALLS];  // lattice type of the wall's nodes: 5/6 slip, 7/8 no-slip (LB.cpp:497-533)
};

namespace hb { struct hb_adj; }

struct hb_ctx {
    hb_params P;
    int X = 0, Y = 0, Z = 0;
    long long N = 0;
    int dev = 0;
    cudaStream_t stream = nullptr;
    size_t sz = 8;              // bytes per stored population
    // lattice
    uint8_t* ntype = nullptr;
    unsigned long long* lmask = nullptr;  // [N] general / static-wall links of non-bulk active nodes (FP32/FP16 kernel)
    uint32_t* solid = nullptr;
    void* fA = nullptr;
    void* fB = nullptr;
    int cur = 0;                // population buffer holding the current state (0: fA, 1: fB)
    int* mode = nullptr;        // device
    double* rho = nullptr;
    double* u = nullptr;
    double* hf = nullptr;
    double* mass = nullptr;
    void* visc = nullptr;
    void* dv = nullptr;
    unsigned long long* hacc = nullptr;  // [7E] fixed-point element sums of the FP32/FP16 kernels
    int* status = nullptr;      // [STATUS_WORDS]
    double* wall_part = nullptr;
    double* wall_force = nullptr;   // [MAX_WALLS*3 + 1]
    int lb_grid = 0, lb_block = 256;
    bool has_dynwall = false;
    bool initialized = false;
    long long steps = 0;
    bool dem_stepped = false;   // a DEM substep has run (particle energies exist)
    double* fs_force = nullptr; // device lbF seen by the free-surface init of new cells
    double* lb_force = nullptr; // device lbF seen by the collision (zero without forceField), 5 doubles:
                                // the FP64 force and, from byte 24, its FP32 copy
    float* lb_force_f = nullptr;    // = (float*)(lb_force + 3), not a separate allocation
    uint8_t* io_linked = nullptr;   // [N] output mirror: wall nodes that own a node object
    void* io_part = nullptr;        // output mirror: per-block partials + result block
    double* io_terms = nullptr;     // output mirror: per-element terms [7E]
    double* d_stage = nullptr;      // device staging of element downloads (35 E doubles)
    double* h_stage = nullptr;      // pinned host staging of element downloads (35 E doubles)
    // free surface
    double* fs_scal = nullptr;      // [0]=surplus [1]=interface count as double
    uint8_t* fs_flag = nullptr;     // per-node conversion flags of the current step
    double* fs_mass2 = nullptr;     // new interface masses (updateMass reads the old ones)
    int* fs_first = nullptr;        // 64-byte step state of the free surface (first-step flag,
                                    // list selector and counts, 128-bit surplus ledger)
    uint32_t* fs_ilist = nullptr;   // [4 fs_icap] two interface lists, conversion list, new cells
    uint32_t* fs_parent = nullptr;  // [N] claim slots of the new interface cells (zero between steps)
    long long fs_icap = 0;          // list capacity (hb_params.cap_interface, 0: every node)
    // cylinders and curved walls (hb_curved.cu)
    std::vector<hb_cyl_host> cyl;
    void* curved_list = nullptr;
    int* curved_cnt = nullptr;
    int curved_n = 0;
    // slip walls (hb_slip.cu)
    unsigned long long* slip_list = nullptr;  // (node, diagonal slip link) entries
    double* slip_val = nullptr;
    uint8_t* slip_mix = nullptr;
    int slip_n = 0;
    // DEM
    hb_dem_dev d;
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // cycle graphs starting from fA / fB
    cudaGraph_t graph2 = nullptr;
    cudaGraphNode_t mask_node[2] = {nullptr, nullptr};  // the mask kernel in graph / graph2 (carries lbF)
    bool force_dirty = false;    // lbF changed through the graphs' nodes, lb_force not yet written
    int mode_val = -1;           // value last written to *mode (-1: unknown)
    bool mirror = true;          // hb_cycle's last step writes every node's rho, u, hydroForce
    bool mirror_valid = true;    // those node fields are the last step's (downloads need them)
    // element sink (hb_set_element_sink): device aliases of mapped host arrays the cycle
    // graphs fill at the end of every cycle, in the order of hb_download_elements
    double* sink[11] = {};
    bool sink_on = false;
    bool reduce_pending = false; // element forces lag the last lattice step
    int kernels_per_cycle = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    hb::hb_adj* adj = nullptr;  // adjoint buffers (checkpoints, tape), allocated on first use
};

// launchers implemented in the .cu files (all enqueue on ctx->stream)
namespace hb {
int launch_init_lattice(hb_ctx* c, const double* el_x0, const double* el_r, int E,
                        const double* ob_x0, const double* ob_r, int O);
void launch_refresh_bulk(hb_ctx* c, int* changed = nullptr);
void launch_lb_step(hb_ctx* c, int cur);
void launch_lb_step_dev(hb_ctx* c, const LBArgs& a);
void launch_lb_wallforce(hb_ctx* c, int cur);
int launch_upload_lattice(hb_ctx* c, const uint8_t* type, const uint8_t* inside,
                          const uint32_t* solid, const double* f, const double* n, const double* u,
                          const double* mass, const double* visc);
int launch_download_lattice(hb_ctx* c, double* f_dev, int which_parity);
int launch_ghosts_init(hb_ctx* c);
int launch_cycle_coop(hb_ctx* c, int do_reduce, int do_dem, int do_boxes, unsigned long long* ts = nullptr);
void launch_couple(hb_ctx* c, bool build_boxes, int cur, cudaEvent_t* ev = nullptr);
cudaGraphNode_t find_mask_node(cudaGraph_t g);
int update_mask_force(hb_ctx* c);
void flush_body_force(hb_ctx* c);  // write lb_force now if the graphs hold a newer lbF
// moving bounce-back (hb_lb.cu): refill of uncovered nodes and link masks after the
// coupling masks; element force and torque after the lattice step
void launch_mbb_nodes(hb_ctx* c, int cur);
void launch_mbb_force(hb_ctx* c, int cur);
void launch_dem_first_predict(hb_ctx* c);
void launch_couple_reduce(hb_ctx* c);
void launch_reactions(hb_ctx* c);
int set_error(int code, const char* msg);  // hb_last_error text, returns code
size_t fs_count_bytes();
void fs_invalidate(hb_ctx* c);  // rebuild the interface list from the node bytes at the next step
void fs_count_for_file(void* rec);  // the step state as a checkpoint holds it (no list)
// curved walls (hb_curved.cu)
void launch_init_cylinders(hb_ctx* c);
int curved_init(hb_ctx* c);
void curved_remark(hb_ctx* c);
void launch_curved(hb_ctx* c, void* f);
// slip walls (hb_slip.cu)
int slip_init(hb_ctx* c);
void launch_slip(hb_ctx* c, void* f);
// output mirror (hb_io.cu)
int io_prepare(hb_ctx* c);
void launch_io_pack(hb_ctx* c, int8_t* type, double* v, double* pressure, double* visc, double* mass,
                    uint32_t* solid);
double* launch_io_export(hb_ctx* c);
int io_slot_count();  // wall / object FParticle of the last substep into d.react
void launch_fs_step(hb_ctx* c, int cur);
int fs_init(hb_ctx* c);
int dem_init(hb_ctx* c, const hb_elements* e, const hb_objects* o);
int dem_args_upload(hb_ctx* c);
int adjoint_run(hb_ctx* c, const hb_adjoint_cfg* cfg, bool reverse, double* J, double* dF, double* dtau,
                double* duin, std::string& err);
int adjoint_timing(hb_ctx* c, float* ms_forward, float* ms_reverse, int64_t* fwd_steps, int64_t* rev_steps);
void adjoint_free(hb_ctx* c);
}  // namespace hb
