// hb_ckpt.cu -- full-state checkpoint / restart of a context, and the reference's
// particle recycle file.
//
// The reference has no lattice restart (its .restart file, DEM.cpp:2337-2420, holds DEM
// metadata only, and exportRecycleParticles writes particle rows at six digits).  A
// checkpoint here is every device buffer that carries state from one step to the next,
// byte for byte, plus the host-side step state; restarting from it continues the run
// bit-identically.  File layout (little-endian, native struct layout):
//   header  "HBCKPT01", uint32 version, uint32 sizeof(hb_params), hb_params,
//           int64 N, E, O, int64 steps, int32 cur, uint8 reduce_pending, dem_stepped
//   records char name[24], uint64 bytes, payload   (the cylinders as given, then the
//           buffers of state_buffers())
// The loader rebuilds the context with hb_create + hb_init from the saved parameters,
// particles and objects (so every allocation and both cycle graphs exist), then
// overwrites each buffer and the host step state.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <locale>
#include <sstream>
#include <string>
#include <vector>

#include "hb_common.cuh"
#include "hb_ctx.h"

namespace {

constexpr char MAGIC[8] = {'H', 'B', 'C', 'K', 'P', 'T', '0', '1'};
constexpr uint32_t VERSION = 2;

struct Buf {
    const char* name;
    void* ptr;
    size_t bytes;
};

struct Header {
    int64_t N, E, O, steps;
    int32_t cur;
    uint8_t reduce_pending, dem_stepped, mirror_valid, pad;
};

// Every buffer whose contents a later step reads.  Scratch that each step rewrites
// before reading (partials, claim lists, staging, output mirror) is left out.
std::vector<Buf> state_buffers(hb_ctx* c) {
    std::vector<Buf> b;
    auto add = [&](const char* n, void* p, size_t bytes) {
        if (p && bytes) b.push_back(Buf{n, p, bytes});
    };
    const size_t N = (size_t)c->N;
    const size_t tsz = c->P.precision == HB_FP64 ? 8 : 4;
    add("ntype", c->ntype, N);
    add("lmask", c->lmask, 8 * N);
    add("solid", c->solid, 4 * N);
    add("f", c->cur ? c->fB : c->fA, 19 * N * c->sz);
    add("rho", c->rho, 8 * N);
    add("u", c->u, 24 * N);
    add("hf", c->hf, 24 * N);
    add("mass", c->mass, 8 * N);
    add("visc", c->visc, N * tsz);
    add("dv", c->dv, 3 * N * tsz);
    add("status", c->status, sizeof(int) * hb::STATUS_WORDS);
    add("wall_force", c->wall_force, sizeof(double) * (hb::MAX_WALLS * 3 + 1));
    add("fs_force", c->fs_force, sizeof(double) * 3);
    add("lb_force", c->lb_force, sizeof(double) * 5);
    if (c->fs_flag) {  // the interface list itself is rebuilt from the node bytes after a load
        add("fs_scal", c->fs_scal, sizeof(double) * 3);
        add("fs_flag", c->fs_flag, N);
        add("fs_mass2", c->fs_mass2, 8 * N);
        add("fs_first", c->fs_first, hb::fs_count_bytes());
    }
    hb_dem_dev& d = c->d;
    const size_t E = (size_t)d.E;
    if (E) {
        add("hacc", c->hacc, 8 * 7 * E);
        add("dem_base", d.base, 8 * (size_t)DEM_FIELDS * E);
        const size_t Pl = (size_t)d.P;  // particles (= elements for single spheres)
        const size_t S = Pl + (size_t)d.gcap;
        add("dem_pf", d.pf, 4 * 12 * (d.gen ? S : E));
        add("dem_plain", d.plain, 4 * E);
        add("cell_of", d.cell_of, 4 * S);
        add("cell_cnt", d.cell_cnt, 4 * (size_t)d.ncells);
        add("cell_start", d.cell_start, 4 * ((size_t)d.ncells + 1));
        add("cell_fill", d.cell_fill, 4 * (size_t)d.ncells);
        add("cell_items", d.cell_items, 4 * S);
        if (d.gen) {  // particles and the ghost particles of the last rebuild
            add("ghost_meta", d.gmeta, 2 * sizeof(int));
            add("ghost_orig", d.gorig, 4 * (size_t)d.gcap);
            add("ghost_vec", d.gvec, 8 * 3 * (size_t)d.gcap);
            add("ghost_comp", d.comp, 4 * 6 * Pl);
            add("ghost_ccnt", d.ccnt, 4 * Pl);
            add("ghost_ecomp", d.ecomp, 4 * 6 * Pl);
            add("ghost_eccnt", d.eccnt, 4 * E);
            add("ghost_px", d.px, 8 * 3 * S);
            add("part_key", d.pkey, 4 * S);
            add("part_cen", d.pcen, 8 * 3 * S);
            add("dem_size", d.esize, 4 * E);
        }
        add("nbr", d.nbr, 4 * Pl * d.nbr_cap);
        add("nbr_pair_constants", d.npc, 8 * 4 * Pl * d.nbr_cap);
        add("nbr_cnt", d.nbr_cnt, 4 * Pl);
        add("wall_of", d.wall_of, 4 * Pl);
        add("obj", d.obj, 4 * Pl * hb::OBJ_CAP);
        add("obj_cnt", d.obj_cnt, 4 * Pl);
        add("dem_scal", d.scal, 8 * 8);
        add("contacts", d.contacts, 4);
        add("cyl_of", d.cyl_of, 4 * Pl);
        add("wrec", d.wrec, 8 * 7 * Pl);
        add("orec", d.orec, 8 * 7 * Pl * hb::OBJ_CAP);
        add("react", d.react, 8 * 3 * ((size_t)hb::MAX_WALLS + d.O));
    }
    if (d.O) {
        add("obj_x0", d.obj_x0, 8 * 3 * (size_t)d.O);
        add("obj_x1", d.obj_x1, 8 * 3 * (size_t)d.O);
        add("obj_r", d.obj_r, 8 * (size_t)d.O);
    }
    return b;
}

int err(int code, const std::string& m) { return hb::set_error(code, m.c_str()); }

template <class T>
bool rd(std::ifstream& f, T* v, size_t n = 1) {
    f.read(reinterpret_cast<char*>(v), sizeof(T) * n);
    return (bool)f;
}

}  // namespace

extern "C" {

int hb_checkpoint_save(hb_ctx* c, const char* path) {
    if (!c || !path || !c->initialized) return err(HB_ERR_ARG, "null argument or not initialised");
    hb::flush_body_force(c);  // the saved lb_force is the current lbF
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return err(HB_ERR_CUDA, "stream synchronize failed");
    std::ofstream f(path, std::ios::binary);
    if (!f) return err(HB_ERR_ARG, std::string("cannot open ") + path);
    const uint32_t ps = sizeof(hb_params);
    f.write(MAGIC, 8);
    f.write(reinterpret_cast<const char*>(&VERSION), 4);
    f.write(reinterpret_cast<const char*>(&ps), 4);
    f.write(reinterpret_cast<const char*>(&c->P), ps);
    Header h = {};
    h.N = c->N; h.E = c->d.E; h.O = c->d.O_std; h.steps = c->steps; h.cur = c->cur;
    h.reduce_pending = c->reduce_pending; h.dem_stepped = c->dem_stepped; h.mirror_valid = c->mirror_valid;
    f.write(reinterpret_cast<const char*>(&h), sizeof(h));
    {  // the cylinders (host data: they define the curved walls the loader rebuilds)
        char nm[24] = "cylinders";
        const uint64_t n = sizeof(hb_cyl_host) * c->cyl.size();
        f.write(nm, 24);
        f.write(reinterpret_cast<const char*>(&n), 8);
        if (n) f.write(reinterpret_cast<const char*>(c->cyl.data()), (std::streamsize)n);
    }
    std::vector<char> host;
    for (const Buf& b : state_buffers(c)) {
        char nm[24] = {};
        strncpy(nm, b.name, 23);
        const uint64_t n = b.bytes;
        host.resize(b.bytes);
        if (cudaMemcpy(host.data(), b.ptr, b.bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            return err(HB_ERR_CUDA, std::string("checkpoint read of ") + b.name);
        if (b.ptr == c->fs_first) hb::fs_count_for_file(host.data());
        f.write(nm, 24);
        f.write(reinterpret_cast<const char*>(&n), 8);
        f.write(host.data(), (std::streamsize)b.bytes);
    }
    if (!f) return err(HB_ERR_ARG, std::string("write failed: ") + path);
    return HB_OK;
}

int hb_checkpoint_load(const char* path, hb_ctx** out) {
    if (!path || !out) return err(HB_ERR_ARG, "null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return err(HB_ERR_ARG, std::string("cannot open ") + path);
    char magic[8];
    uint32_t ver = 0, ps = 0;
    if (!rd(f, magic, 8) || memcmp(magic, MAGIC, 8) || !rd(f, &ver) || ver != VERSION || !rd(f, &ps) ||
        ps != sizeof(hb_params))
        return err(HB_ERR_ARG, "not a checkpoint of this library version");
    hb_params P;
    Header h;
    if (!rd(f, &P) || !rd(f, &h)) return err(HB_ERR_ARG, "truncated checkpoint header");
    // read every record first: the particles and objects of the saved state define the
    // context that hb_init builds
    std::vector<std::string> names;
    std::vector<std::vector<char>> data;
    while (true) {
        char nm[24];
        uint64_t n = 0;
        if (!f.read(nm, 24)) break;
        if (!rd(f, &n)) return err(HB_ERR_ARG, "truncated checkpoint record");
        names.emplace_back(nm, strnlen(nm, 24));
        data.emplace_back(n);
        if (!f.read(data.back().data(), (std::streamsize)n)) return err(HB_ERR_ARG, "truncated checkpoint record");
    }
    auto find = [&](const char* n) -> const std::vector<char>* {
        for (size_t k = 0; k < names.size(); ++k)
            if (names[k] == n) return &data[k];
        return nullptr;
    };
    const int E = (int)h.E, O = (int)h.O;
    std::vector<double> rad, x0, x1, w0, q0, ox0, ox1, orad;
    std::vector<int32_t> esz;
    hb_elements el = {};
    hb_objects ob = {};
    if (E > 0) {
        const std::vector<char>* base = find("dem_base");
        if (!base || base->size() != 8 * (size_t)DEM_FIELDS * E) return err(HB_ERR_ARG, "checkpoint lacks the element state");
        const double* b = reinterpret_cast<const double*>(base->data());
        // field offsets of hb_dem_dev::base (see DEM_FIELDS): x[0] at 0, x[1] at 3E,
        // w[0] at 36E, q[0] at 72E, rad last
        auto field = [&](size_t off, size_t comps) {
            return std::vector<double>(b + off * E, b + (off + comps) * E);
        };
        x0 = field(0, 3); x1 = field(3, 3); w0 = field(36, 3); q0 = field(72, 4);
        rad = field((size_t)DEM_FIELDS - 1, 1);
        el.count = E;
        el.radius = rad.data(); el.x0 = x0.data(); el.x1 = x1.data(); el.w0 = w0.data(); el.q0 = q0.data();
        if (const std::vector<char>* sz = find("dem_size")) {  // multi-sphere elements
            if (sz->size() != 4 * (size_t)E) return err(HB_ERR_ARG, "checkpoint element sizes of another count");
            esz.assign(reinterpret_cast<const int32_t*>(sz->data()), reinterpret_cast<const int32_t*>(sz->data()) + E);
            el.size = esz.data();
        }
    }
    int Ot = 0;  // objects including the periodic images the loader's init appends again
    if (O > 0) {
        const std::vector<char>* a = find("obj_x0"), *v = find("obj_x1"), *r = find("obj_r");
        if (!a || !v || !r) return err(HB_ERR_ARG, "checkpoint lacks the objects");
        Ot = (int)(r->size() / sizeof(double));
        if (Ot < O || a->size() != 24 * (size_t)Ot || v->size() != 24 * (size_t)Ot)
            return err(HB_ERR_ARG, "checkpoint object records of another size");
        const double* pa = reinterpret_cast<const double*>(a->data());
        const double* pv = reinterpret_cast<const double*>(v->data());
        ox0.resize(3 * (size_t)O);
        ox1.resize(3 * (size_t)O);
        for (int q = 0; q < 3; ++q)
            for (int k = 0; k < O; ++k) {
                ox0[(size_t)q * O + k] = pa[(size_t)q * Ot + k];
                ox1[(size_t)q * O + k] = pv[(size_t)q * Ot + k];
            }
        orad.assign(reinterpret_cast<const double*>(r->data()), reinterpret_cast<const double*>(r->data()) + O);
        ob.count = O; ob.radius = orad.data(); ob.x0 = ox0.data(); ob.x1 = ox1.data();
    }
    hb_ctx* c = nullptr;
    int rc = hb_create(&P, &c);
    if (rc) return rc;
    if (const std::vector<char>* cy = find("cylinders")) {
        const size_t nc = cy->size() / sizeof(hb_cyl_host);
        c->cyl.assign(reinterpret_cast<const hb_cyl_host*>(cy->data()),
                      reinterpret_cast<const hb_cyl_host*>(cy->data()) + nc);
    }
    rc = hb_init(c, E > 0 ? &el : nullptr, O > 0 ? &ob : nullptr);
    if (rc) { hb_destroy(c); return rc; }
    if (c->N != h.N || c->d.E != E || c->d.O != Ot) {
        hb_destroy(c);
        return err(HB_ERR_ARG, "checkpoint sizes do not match the rebuilt context");
    }
    c->cur = h.cur;  // selects the population buffer that "f" restores
    for (const Buf& b : state_buffers(c)) {
        const std::vector<char>* src = find(b.name);
        if (!src || src->size() != b.bytes) {
            hb_destroy(c);
            return err(HB_ERR_ARG, std::string("checkpoint record missing or of another size: ") + b.name);
        }
        if (cudaMemcpy(b.ptr, src->data(), b.bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
            hb_destroy(c);
            return err(HB_ERR_CUDA, std::string("checkpoint restore of ") + b.name);
        }
    }
    hb::fs_invalidate(c);
    c->steps = h.steps;
    c->reduce_pending = h.reduce_pending != 0;
    c->dem_stepped = h.dem_stepped != 0;
    c->mirror_valid = h.mirror_valid != 0;
    if (c->io_part) {  // output-mirror marks are rebuilt from the restored types on demand
        cudaFree(c->io_linked);
        cudaFree(c->io_part);
        cudaFree(c->io_terms);
        c->io_linked = nullptr;
        c->io_part = nullptr;
        c->io_terms = nullptr;
    }
    *out = c;
    return HB_OK;
}

// IO::exportRecycleParticles (IO.cpp:486-535): element count, then per element index,
// size, radius, x0 (moved back into the box through the periodic faces), x1, w0, q0, q1
// with default stream formatting.
int hb_write_recycle_particles(hb_ctx* c, const char* path) {
    if (!c || !path || !c->initialized) return err(HB_ERR_ARG, "null argument or not initialised");
    const int E = c->d.E;
    std::vector<double> b((size_t)DEM_FIELDS * (E > 0 ? E : 1));
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return err(HB_ERR_CUDA, "stream synchronize failed");
    if (E > 0 && cudaMemcpy(b.data(), c->d.base, 8 * (size_t)DEM_FIELDS * E, cudaMemcpyDeviceToHost) != cudaSuccess)
        return err(HB_ERR_CUDA, "element download failed");
    std::ofstream f(path);
    if (!f) return err(HB_ERR_ARG, std::string("cannot open ") + path);
    f.imbue(std::locale::classic());
    std::vector<int> esz(E > 0 ? E : 1, 1);
    if (E > 0 && c->d.esize && cudaMemcpy(esz.data(), c->d.esize, sizeof(int) * E, cudaMemcpyDeviceToHost) != cudaSuccess)
        return err(HB_ERR_CUDA, "element size download failed");
    f << (size_t)E << "\n";
    auto at = [&](size_t off, int k, int i) { return b[(off + k) * E + i]; };
    for (int i = 0; i < E; ++i) {
        f << i << " " << esz[i] << " " << at((size_t)DEM_FIELDS - 1, 0, i) << " ";
        double x[3] = {at(0, 0, i), at(0, 1, i), at(0, 2, i)}, pp[3] = {x[0], x[1], x[2]};
        for (int bb = 0; bb < c->d.npbc; ++bb) {  // pbc planes (utils.cpp:240-245)
            const double* v = c->d.pbc_v[bb];
            const double* p1 = c->d.pbc_p[bb];
            const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const double n1[3] = {v[0] / nv, v[1] / nv, v[2] / nv};
            const double ld = n1[0] * (x[0] - p1[0]) + n1[1] * (x[1] - p1[1]) + n1[2] * (x[2] - p1[2]);
            const double rd = (-1.0 * n1[0]) * (x[0] - (p1[0] + v[0])) + (-1.0 * n1[1]) * (x[1] - (p1[1] + v[1])) +
                              (-1.0 * n1[2]) * (x[2] - (p1[2] + v[2]));
            if (ld < 0.0) for (int k = 0; k < 3; ++k) pp[k] = pp[k] + v[k];
            if (rd < 0.0) for (int k = 0; k < 3; ++k) pp[k] = pp[k] - v[k];
        }
        for (int k = 0; k < 3; ++k) f << pp[k] << " ";   // x0
        for (int k = 0; k < 3; ++k) f << at(3, k, i) << " ";   // x1
        for (int k = 0; k < 3; ++k) f << at(36, k, i) << " ";  // w0
        for (int k = 0; k < 4; ++k) f << at(72, k, i) << " ";  // q0
        for (int k = 0; k < 4; ++k) f << at(76, k, i) << (k == 3 ? "\n" : " ");  // q1
    }
    if (!f) return err(HB_ERR_ARG, std::string("write failed: ") + path);
    return HB_OK;
}

}  // extern "C"
