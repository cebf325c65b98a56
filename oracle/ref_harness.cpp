// Test infrastructure only: drives the reference hybird code, built from its own
// unmodified sources, and dumps its full FP64 state so the parity fixtures under
// tests/golden/ can be generated from the reference itself.  Nothing in the product
// links or calls this file.
//
// Usage:  ref_dump <config.cfg> <workdir> <out.bin> <step> [<step> ...] [--gasbox fx fz] [--vtk]
//                  [--cylinder p1x p1y p1z p2x p2y p2z R]
//
// The driver mirrors hybird.cpp:245-344 (main): parseCommandLine -> parseConfigFile ->
// io.initialize -> lb.latticeDefinition -> dem.discreteElementInit ->
// lb.latticeBolzmannInit -> goCycle x N (hybird.cpp:35-66).  After each requested
// step count the state is appended to <out.bin> as named records.
//
// --cylinder adds one static cylinder to dem.cylinders after dem.discreteElementInit (as
// the DRUM/AVALANCHE/NET problem cases do, DEM.cpp:871-935, without their other
// settings), so the lattice initialisation marks curved walls around it.
//
// --gasbox fx fz replaces lb.latticeBolzmannInit by its pieces (LB.cpp:190-219,
// 324-340) and marks gas where x >= fx*lbSizeX or z >= fz*lbSizeZ before the generic
// interface loops (LB.cpp:787-814) run; this is the dam-break column used for the
// free-surface fixtures, for which the reference has no problemName case.
//
// Besides the state, each record set holds the reference's own output-step quantities:
// objects[].FParticle, the IO data-elaboration functions (IO.cpp:969-1106) and, with
// --vtk, the text IO::exportParaviewFluidOld writes (IO.cpp:698-831) and the particle
// recycle file of IO::exportRecycleParticles (IO.cpp:486-535).

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <string>
#include <vector>
#include <fstream>
#include <iostream>
#include <iomanip>
#include <sstream>
#include <algorithm>
#include <ctime>
#include <csignal>
#include <sys/stat.h>

#define private public
#define protected public
#include "IO.h"
#include "DEM.h"
#include "LB.h"
#undef private
#undef protected

void parseCommandLine(IO& io, GetPot& command_line);
void parseConfigFile(IO& io, DEM& dem, LB& lb, GetPot& lbmCfgFile, GetPot& command_line);
void goCycle(IO& io, DEM& dem, LB& lb);

namespace {

FILE* g_out = nullptr;
bool g_vtk = false;
bool g_cyl = false;
double g_cylv[7] = {0, 0, 0, 0, 0, 0, 0};
std::string g_work;

// record: char name[32]; uint32 dtype (0=f64,1=u32,2=u8,3=i64); uint64 count; payload
void put(const char* name, uint32_t dtype, uint64_t count, const void* data, size_t esz) {
    char nm[32];
    memset(nm, 0, sizeof(nm));
    strncpy(nm, name, 31);
    fwrite(nm, 1, 32, g_out);
    fwrite(&dtype, 4, 1, g_out);
    fwrite(&count, 8, 1, g_out);
    if (count) fwrite(data, esz, count, g_out);
}
void put_f64(const char* n, const std::vector<double>& v) { put(n, 0, v.size(), v.data(), 8); }
void put_u32(const char* n, const std::vector<uint32_t>& v) { put(n, 1, v.size(), v.data(), 4); }
void put_u8(const char* n, const std::vector<uint8_t>& v) { put(n, 2, v.size(), v.data(), 1); }
void put_i64(const char* n, const std::vector<int64_t>& v) { put(n, 3, v.size(), v.data(), 8); }

void vec3(std::vector<double>& out, const tVect& a) {
    out.push_back(a.x); out.push_back(a.y); out.push_back(a.z);
}

void dump(IO& io, DEM& dem, LB& lb, long step) {
    const size_t N = io.lbmSolve ? lb.totNodes : 0;
    std::vector<int64_t> hdr = {step, (int64_t)lb.lbSize[0], (int64_t)lb.lbSize[1],
                                (int64_t)lb.lbSize[2], (int64_t)lb.activeNodes.size(),
                                (int64_t)dem.elmts.size(), (int64_t)dem.multiStep};
    put_i64("header", hdr);
    std::vector<uint8_t> type(N), inside(N), has(N);
    if (N) {
    std::vector<uint32_t> solid(N);
    std::vector<double> f(19 * N, 0.0), fs(19 * N, 0.0), n(N, 0.0), u(3 * N, 0.0),
        mass(N, 0.0), visc(N, 0.0), hf(3 * N, 0.0);
    for (size_t i = 0; i < N; ++i) {
        type[i] = (uint8_t)lb.types[i].getType();
        inside[i] = lb.types[i].isInsideParticle() ? 1 : 0;
        solid[i] = lb.types[i].getSolidIndex();
        node* nd = lb.nodes[i];
        has[i] = nd ? 1 : 0;
        if (!nd) continue;
        for (int j = 0; j < 19; ++j) {
            f[j * N + i] = nd->f[j];
            fs[j * N + i] = nd->fs[j];
        }
        n[i] = nd->n;
        u[0 * N + i] = nd->u.x; u[1 * N + i] = nd->u.y; u[2 * N + i] = nd->u.z;
        mass[i] = nd->mass;
        visc[i] = nd->visc;
        hf[0 * N + i] = nd->hydroForce.x; hf[1 * N + i] = nd->hydroForce.y;
        hf[2 * N + i] = nd->hydroForce.z;
    }
    put_u8("type", type); put_u8("inside", inside); put_u8("has_node", has);
    put_u32("solid", solid);
    put_f64("f", f); put_f64("fs", fs); put_f64("n", n); put_f64("u", u);
    put_f64("mass", mass); put_f64("visc", visc); put_f64("hydroForce", hf);
    std::vector<uint32_t> il(lb.interfaceNodes.begin(), lb.interfaceNodes.end());
    put_u32("interfaceNodes", il);
    std::vector<uint32_t> pl(lb.particleNodes.begin(), lb.particleNodes.end());
    put_u32("particleNodes", pl);
    std::vector<double> sc = {lb.totalMass};
    put_f64("totalMass", sc);
    }

    // DEM state (FP64, physical units == lattice units for unit=1 configs)
    std::vector<double> ex0, ex1, ex2, ew, eq, efh, emh, efp, efw, emp, emw, evol, em, eI;
    for (auto& e : dem.elmts) {
        vec3(ex0, e.x0); vec3(ex1, e.x1); vec3(ex2, e.x2); vec3(ew, e.wGlobal);
        eq.push_back(e.q0.q0); eq.push_back(e.q0.q1); eq.push_back(e.q0.q2); eq.push_back(e.q0.q3);
        vec3(efh, e.FHydro); vec3(emh, e.MHydro); vec3(efp, e.FParticle); vec3(efw, e.FWall);
        vec3(emp, e.MParticle); vec3(emw, e.MWall);
        evol.push_back(e.fluidVolume); em.push_back(e.m); vec3(eI, e.I);
    }
    put_f64("e_x0", ex0); put_f64("e_x1", ex1); put_f64("e_x2", ex2); put_f64("e_w", ew);
    put_f64("e_q0", eq); put_f64("e_FHydro", efh); put_f64("e_MHydro", emh);
    put_f64("e_FParticle", efp); put_f64("e_FWall", efw); put_f64("e_MParticle", emp);
    put_f64("e_MWall", emw); put_f64("e_fluidVolume", evol); put_f64("e_m", em); put_f64("e_I", eI);
    std::vector<uint32_t> nt(dem.neighborTable.begin(), dem.neighborTable.end());
    put_u32("neighborTable", nt);
    // ghost particles of the periodic faces (DEM.cpp:1586-1664): origin and shift
    std::vector<uint32_t> gi;
    std::vector<double> gv;
    for (auto& gh : dem.ghosts) { gi.push_back(gh.ghostIndex); vec3(gv, gh.pbcVector); }
    put_u32("ghost_index", gi);
    put_f64("ghost_vec", gv);
    std::vector<uint32_t> nw(dem.nearWallTable.begin(), dem.nearWallTable.end());
    put_u32("nearWallTable", nw);
    std::vector<uint32_t> no(dem.nearObjectTable.begin(), dem.nearObjectTable.end());
    put_u32("nearObjectTable", no);
    std::vector<double> wf;
    for (auto& w : dem.walls) { vec3(wf, w.FHydro); }
    put_f64("w_FHydro", wf);
    std::vector<double> wp;
    for (auto& w : dem.walls) { vec3(wp, w.FParticle); }
    put_f64("w_FParticle", wp);
    std::vector<double> dm = {dem.demTime, dem.maxDisp, dem.nebrRange, dem.deltat,
                              dem.cellWidth[0], dem.cellWidth[1], dem.cellWidth[2],
                              (double)dem.nCells[0], (double)dem.nCells[1], (double)dem.nCells[2],
                              dem.particleEnergy.trKin, dem.particleEnergy.rotKin,
                              dem.particleEnergy.grav};
    put_f64("dem_scalars", dm);
    std::vector<double> of;
    for (auto& o : dem.objects) { vec3(of, o.FParticle); }
    put_f64("o_FParticle", of);

    // IO::outputStep quantities (IO.cpp:132-198).  The two maximum-speed lines
    // (IO.cpp:835-876) only print, so their maxima are taken here the same way.
    double maxFluid = 0.0;
    int64_t active = 0;
    for (size_t i = 0; i < N; ++i)
        if (lb.types[i].isActive()) {
            maxFluid = std::max(maxFluid, lb.nodes[i]->u.norm2());
            ++active;
        }
    double maxPart = 0.0, maxSpin = 0.0;
    for (auto& e : dem.elmts) {
        maxPart = std::max(maxPart, e.x1.norm2());
        maxSpin = std::max(maxSpin, e.wGlobal.norm2());
    }
    const tVect objF = io.totForceObject(dem.objects);
    std::vector<double> iv = {
        sqrt(maxFluid), N ? io.totFluidMass(lb) : 0.0, (N && active) ? io.totPlastic(lb) : 0.0, (double)active,
        sqrt(maxPart), sqrt(maxSpin), io.collisionForceTot(dem.elmts), io.hydraulicForceTot(dem.elmts),
        io.totParticleMass(dem.elmts), objF.x, objF.y, objF.z,
        dem.particleEnergy.kin, dem.particleEnergy.rotKin, dem.particleEnergy.trKin,
        dem.particleEnergy.grav, dem.particleEnergy.total};
    put_f64("io_values", iv);
    if (g_vtk && N) {
        const std::string path = g_work + "/fluid_dump.vti";
        io.exportParaviewFluidOld(lb, path);
        std::ifstream in(path, std::ios::binary);
        std::string txt((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        std::vector<uint8_t> bytes(txt.begin(), txt.end());
        put_u8("vtk", bytes);
    }
    if (g_vtk && !dem.elmts.empty()) {  // IO::exportRecycleParticles (IO.cpp:486-535)
        io.exportRecycleParticles(dem.elmts, dem.pbcs);
        std::stringstream ss;
        ss << io.partDirectory << "/recycle_" << io.currentTimeStep << ".dat";
        std::ifstream in(ss.str(), std::ios::binary);
        std::string txt((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        std::vector<uint8_t> bytes(txt.begin(), txt.end());
        put_u8("recycle", bytes);
    }
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s cfg workdir out.bin step [step...] [--gasbox fx fz]\n", argv[0]);
        return 2;
    }
    std::string cfg = argv[1], work = argv[2], outp = argv[3];
    g_work = work;
    std::vector<long> steps;
    bool gasbox = false;
    double gfx = 1.0, gfz = 1.0;
    for (int a = 4; a < argc; ++a) {
        if (!strcmp(argv[a], "--vtk")) {
            g_vtk = true;
        } else if (!strcmp(argv[a], "--cylinder") && a + 7 < argc) {
            g_cyl = true;
            for (int k = 0; k < 7; ++k) g_cylv[k] = atof(argv[a + 1 + k]);
            a += 7;
        } else if (!strcmp(argv[a], "--gasbox") && a + 2 < argc) {
            gasbox = true;
            gfx = atof(argv[a + 1]);
            gfz = atof(argv[a + 2]);
            a += 2;
        } else {
            steps.push_back(atol(argv[a]));
        }
    }
    std::sort(steps.begin(), steps.end());

    IO io;
    DEM dem;
    LB lb;
    time_t t = time(0);
    io.now = localtime(&t);
    const char* av[] = {"ref_dump", "-c", cfg.c_str(), "-d", work.c_str()};
    GetPot command_line(5, const_cast<char**>(av));
    parseCommandLine(io, command_line);
    GetPot lbmCfgFile(io.lbmCfgName.c_str());
    parseConfigFile(io, dem, lb, lbmCfgFile, command_line);
    io.currentTimeStep = 0;
    io.initialize();
    lb.latticeDefinition();
    dem.discreteElementInit(lb.boundary, lb.lbSize, lb.unit, lb.lbF);
    if (g_cyl) {
        cylinder cy;
        cy.index = (unsigned int)dem.cylinders.size();
        cy.p1 = tVect(g_cylv[0], g_cylv[1], g_cylv[2]);
        cy.p2 = tVect(g_cylv[3], g_cylv[4], g_cylv[5]);
        cy.R = g_cylv[6];
        cy.omega.reset();
        cy.initAxes();
        cy.moving = false;
        cy.slip = false;
        dem.cylinders.push_back(cy);
    }
    if (io.lbmSolve) {
        if (!gasbox) {
            lb.latticeBolzmannInit(dem.cylinders, dem.walls, dem.particles, dem.objects);
        } else {
            // LB.cpp:190-219 with the column geometry injected before the interface loops
            lb.initializeNodes();
            lb.initializeLatticeBoundaries();
            lb.initializeParticleBoundaries(dem.particles);
            lb.initializeWallBoundaries(dem.walls);
            lb.initializeCylinderBoundaries(dem.cylinders);
            lb.initializeObjectBoundaries(dem.objects);
            lb.initializeCurved(dem.cylinders);
            const double xlim = gfx * lb.lbSize[0], zlim = gfz * lb.lbSize[2];
            for (unsigned int it = 0; it < lb.totNodes; ++it) {
                if (lb.types[it].isFluid()) {
                    if (lb.getX(it) >= xlim || lb.getZ(it) >= zlim) lb.types[it].setGas();
                }
            }
            lb.initializeInterface(dem.particles.size());
            lb.initializeLists();
            lb.initializeVariables();
            lb.initializeWalls(dem.walls, dem.cylinders, dem.objects);
            lb.cleanLists();
            lb.totalMass = 0.0;
            for (unsigned int it = 0; it < lb.nodes.size(); ++it) {
                if (lb.types[it].isActive() && !lb.types[it].isInsideParticle())
                    lb.totalMass += lb.nodes[it]->mass;
            }
        }
    }
    lb.time = 0;
    dem.demTime = 0.0;
    dem.demTimeStep = 0;

    g_out = fopen(outp.c_str(), "wb");
    if (!g_out) { perror("open out"); return 3; }
    long done = 0;
    for (long s : steps) {
        while (done < s) {
            goCycle(io, dem, lb);
            ++done;
        }
        dump(io, dem, lb, done);
    }
    fclose(g_out);
    return 0;
}
