// TEST INFRASTRUCTURE ONLY -- CPU FP64 restatement of hybird's time-step path.
//
// Every function names the reference file:line it restates.  Arithmetic is written in
// the reference's evaluation order (left-to-right tVect/tMat operator chains), so on
// one thread it reproduces the reference bit-for-bit; the CUDA library is checked
// against it and against the reference fixtures in tests/golden/.  Parallel loops
// mirror the reference's own OpenMP loops; order-dependent sums (wall forces, mass
// surplus, element forces) run sequentially in the reference's 1-thread order.
//
// Restated here but not present in the reference: TRT collision (two relaxation times
// with a magic parameter), used only where hb_params.collision == HB_TRT.

#include "hb_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

// ---- D3Q19 lattice constants (lattice.h:36-101) -------------------------------------
const int Q = 19;
const int CX[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CY[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0};
const int CZ[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
const int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

int dir_of(int x, int y, int z) {
    for (int j = 0; j < Q; ++j)
        if (CX[j] == x && CY[j] == y && CZ[j] == z) return j;
    return -1;
}
// Slip-wall partners of a diagonal direction j (the lattice.h:87-94 tables): along each of
// j's two non-zero axes, the neighbour one step along that axis and the direction j with
// that component reversed -- the population that, reflected off a wall normal to the
// other axis, arrives as opp(j).  Which axis is "1" does not matter: the rule uses the
// one open side.
struct SlipPair { int check[2], dir[2]; };
SlipPair slip_pair(int j) {
    SlipPair r{{0, 0}, {0, 0}};
    const int c[3] = {CX[j], CY[j], CZ[j]};
    int k = 0;
    for (int a = 0; a < 3 && k < 2; ++a) {
        if (!c[a]) continue;
        int u[3] = {0, 0, 0}, f[3] = {c[0], c[1], c[2]};
        u[a] = c[a];
        f[a] = -c[a];
        r.check[k] = dir_of(u[0], u[1], u[2]);
        r.dir[k] = dir_of(f[0], f[1], f[2]);
        ++k;
    }
    return r;
}
const double W[Q] = {12.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0,
                     2.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                     1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                     1.0 / 36.0};
const double MIN_TAU = 0.501, MAX_TAU = 1.8;  // lattice.h:29-30

struct V3 {
    double x, y, z;
};
inline V3 v3(double a, double b, double c) { return V3{a, b, c}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mul(double s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }  // scalar*vec (vector.cpp)
inline V3 divs(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // vector.cpp:113
inline double norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 cross(V3 a, V3 b) {  // vector.cpp:121-126
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 cvec(int j) { return v3(CX[j], CY[j], CZ[j]); }

struct Quat {
    double q0, q1, q2, q3;
};
inline Quat qmul(Quat a, Quat b) {  // quaternion::multiply, vector.cpp:222-228 (a.multiply(b))
    return Quat{b.q0 * a.q0 - b.q1 * a.q1 - b.q2 * a.q2 - b.q3 * a.q3,
                b.q0 * a.q1 + b.q1 * a.q0 - b.q2 * a.q3 + b.q3 * a.q2,
                b.q0 * a.q2 + b.q1 * a.q3 + b.q2 * a.q0 - b.q3 * a.q1,
                b.q0 * a.q3 - b.q1 * a.q2 + b.q2 * a.q1 + b.q3 * a.q0};
}
inline Quat qadj(Quat a) { return Quat{a.q0, -a.q1, -a.q2, -a.q3}; }
inline Quat qadd(Quat a, Quat b) { return Quat{a.q0 + b.q0, a.q1 + b.q1, a.q2 + b.q2, a.q3 + b.q3}; }
inline Quat qsub(Quat a, Quat b) { return Quat{a.q0 - b.q0, a.q1 - b.q1, a.q2 - b.q2, a.q3 - b.q3}; }
inline Quat qscale(Quat a, double s) { return Quat{a.q0 * s, a.q1 * s, a.q2 * s, a.q3 * s}; }
inline void qnormalize(Quat& a) {  // vector.cpp:196-202
    double nn = std::sqrt(a.q0 * a.q0 + a.q1 * a.q1 + a.q2 * a.q2 + a.q3 * a.q3);
    a.q0 /= nn; a.q1 /= nn; a.q2 /= nn; a.q3 /= nn;
}
inline V3 project(V3 vec, Quat q) {  // vector.cpp:364-370
    Quat vq{0.0, vec.x, vec.y, vec.z};
    Quat r = qmul(qmul(q, vq), qadj(q));
    return v3(r.q1, r.q2, r.q3);
}
inline V3 newtonAcc(V3 m, V3 I, V3 w) {  // vector.cpp:371-376
    return v3((m.x + (I.y - I.z) * w.y * w.z) / I.x, (m.y + (I.z - I.x) * w.z * w.x) / I.y,
              (m.z + (I.x - I.y) * w.x * w.y) / I.z);
}

struct Wall {  // utils.h:18-82, built by DEM::initializeWalls (DEM.cpp:435-633)
    V3 p, n;
    bool moving;
    bool slip = false;
    V3 vel, omega, rot;
    V3 fhydro, fparticle;
    double dist(V3 pt) const { return dot(n, sub(pt, p)); }  // utils.cpp:12-15
    V3 speed(V3 pt) const {                                    // utils.cpp:36-49
        if (!moving) return v3(0, 0, 0);
        V3 dc = sub(pt, rot);
        V3 da = sub(dc, mul(dot(dc, n), n));
        return add(vel, cross(omega, da));
    }
};

struct Elmt {  // elmt.h:53-135
    double radius, m;
    int size;
    V3 I;
    V3 x0, x1, x2, x3, x4, x5, xp0, xp1, xp2, xp3, xp4, xp5;
    Quat q0, q1, q2, q3, q4, q5, qp0, qp1, qp2, qp3, qp4, qp5;
    V3 w0, w1, w2, w3, w4, w5, wp0, wp1, wp2, wp3, wp4, wp5;
    V3 wGlobal, wLocal, wpGlobal, wpLocal;
    V3 FHydro, FParticle, FWall, MHydro, MParticle, MWall;
    double fluidVolume;
};

struct Part {  // particle (elmt.h:137-187): one sphere of an element, or a ghost copy of one
    unsigned cluster;
    int proto;
    double r;
    V3 x0, x1, radiusVec;
};

struct Ghost {  // elmt.h:189-197
    unsigned index;
    V3 vec;
};

struct Pbc {  // utils.h:144-163: base point, shift and the two planes (pbc::setPlanes)
    V3 p, v;
    V3 p1, n1, p2, n2;
    double dist1(V3 x) const { return dot(n1, sub(x, p1)); }
    double dist2(V3 x) const { return dot(n2, sub(x, p2)); }
};

// prototypes of the multi-sphere elements, radius units (DEM::compositeProperties,
// DEM.cpp:404-433; "-1/2" there is an integer division)
V3 prototype(int size, int k) {
    if (size == 2) return k == 0 ? v3(0.5, 0.0, 0.0) : v3(-0.5, 0.0, 0.0);
    if (size == 3) {
        if (k == 0) return v3(0.0, 1.0, 0.0);
        return k == 1 ? v3(-std::sqrt(3.0) / 2, -1 / 2, 0.0) : v3(std::sqrt(3.0) / 2, -1 / 2, 0.0);
    }
    if (size == 4) {
        if (k == 0) return v3(0.0, 0.0, 1.0);
        if (k == 1) return v3(0.0, 2.0 * std::sqrt(2.0) / 3.0, -1.0 / 3.0);
        if (k == 2) return v3(2.0 * std::sqrt(6.0) / 6.0, -2.0 * std::sqrt(2.0) / 6.0, -1.0 / 3.0);
        return v3(-2.0 * std::sqrt(6.0) / 6.0, -2.0 * std::sqrt(2.0) / 6.0, -1.0 / 3.0);
    }
    return v3(0.0, 0.0, 0.0);
}

struct Cyl {  // utils.h:85-110 (cylinder), initAxes utils.cpp:154-161
    V3 p1, p2, naxes, omega;
    double R;
    bool moving;
};

// tinyVector::insideCylinder (vector.cpp:160-170)
bool insideCylinder(const V3& pt, const V3& p1, const V3& naxes, double R) {
    const V3 d = sub(pt, p1);
    const V3 ax = mul(dot(d, naxes), naxes);
    return norm2(sub(d, ax)) < R * R;
}
// cylinder::getSpeed (utils.cpp:106-120)
V3 cylinderSpeed(const Cyl& c, const V3& pt) {
    if (!c.moving) return v3(0.0, 0.0, 0.0);
    const V3 pt1 = sub(pt, c.p1);
    const V3 proj = add(c.p1, mul(dot(c.naxes, pt1), c.naxes));
    return cross(c.omega, sub(pt, proj));
}
// cylinder::segmentIntercept (utils.cpp:177-224), both roots with -sqrt as the reference
double segmentIntercept(const Cyl& c, const V3& start, const V3& dir) {
    const V3 AB = sub(c.p2, c.p1);
    const V3 AO = sub(start, c.p1);
    const V3 AOxAB = cross(AO, AB);
    const V3 VxAB = cross(dir, AB);
    const double ab2 = dot(AB, AB);
    const double a = dot(VxAB, VxAB);
    const double b = 2 * dot(VxAB, AOxAB);
    const double cc = dot(AOxAB, AOxAB) - (c.R * c.R * ab2);
    const double disc = b * b - 4 * a * cc;
    if (disc < 0) return 0.0;
    const double t1 = (-b - std::sqrt(disc)) / (2 * a);
    if (t1 < 0) return 0.0;
    return t1;
}
// cylinder::dist (utils.cpp:56-67): distance of a point from the cylinder surface
double cylinderDist(const Cyl& c, const V3& pt) {
    const V3 d = sub(pt, c.p1);
    const V3 ax = mul(dot(d, c.naxes), c.naxes);
    return c.R - std::sqrt(norm2(sub(ax, d)));
}
// cylinder::vecDist (utils.cpp:69-82)
V3 cylinderVecDist(const Cyl& c, const V3& pt) {
    const V3 proj = add(c.p1, mul(dot(c.naxes, sub(pt, c.p1)), c.naxes));
    const V3 dfa = sub(pt, proj);
    return sub(pt, add(proj, mul(c.R, divs(dfa, std::sqrt(norm2(dfa))))));
}

struct Object {  // elmt.h:199-221
    double r;
    V3 x0, x1, fparticle;
};

}  // namespace

struct hbo_sim {
    hb_params P;
    int X, Y, Z;
    size_t N;
    int periodic[6];
    // node state (node.h:17-46) in structure-of-arrays form
    std::vector<uint8_t> type, inside, has;
    std::vector<uint32_t> solid;
    std::vector<uint32_t> nb;  // neighbor table d[i*19+j] (LB.cpp:370-473)
    std::vector<double> f, fs;  // [i*19+j]
    std::vector<double> n, mass, newMass, visc;
    std::vector<V3> u, hf;
    std::vector<uint32_t> fluidNodes, interfaceNodes, particleNodes, activeNodes;
    V3 lbF;
    double totalMass;
    // DEM
    std::vector<Elmt> el;
    std::vector<Part> parts;                   // standard particles, then ghosts
    unsigned stdParticles = 0;
    std::vector<std::vector<unsigned>> comps;  // per element: its particles, ghosts appended
    std::vector<Pbc> pbcs;
    std::vector<Ghost> ghosts;
    unsigned stdObjects = 0;
    bool newNeighborList = false;
    std::vector<Object> obj;
    std::vector<Wall> walls;
    std::vector<Cyl> cyl;
    std::vector<double> delta;  // [i*19+j] curve::delta of curved nodes (LB.cpp:589-603)
    V3 demF;
    double deltat, demTime, maxDisp, nebrRange, trigger;
    bool triggerSet;
    double cellWidth[3];
    unsigned nCells[3];
    double dampCoeff, knConst, ksConst;
    std::vector<int> cellTable;
    std::vector<uint32_t> neighborTable, nearWallTable, nearObjectTable, nearCylinderTable;
    std::vector<int> tableCell;

    size_t idx(int x, int y, int z) const { return (size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z); }
    int gx(size_t i) const { return (int)(i % X); }
    int gy(size_t i) const { return (int)((i / X) % Y); }
    int gz(size_t i) const { return (int)(i / ((size_t)X * Y)); }
    V3 pos(size_t i) const { return v3(gx(i), gy(i), gz(i)); }
    bool isActive(size_t i) const { return type[i] == 0 || type[i] == 3; }
    bool isWall(size_t i) const { return type[i] >= 5 && type[i] <= 9; }
};

namespace {

bool fail(const char* msg) {
    g_err = msg;
    return false;
}

// node::initialize + setEquilibrium (node.cpp:26-61)
void nodeInit(hbo_sim& s, size_t i, double density, V3 vel, double massF, double viscosity, V3 F) {
    s.n[i] = density;
    s.mass[i] = massF;
    V3 half = divs(divs(mul(1.0, F), 2.0), density);
    s.u[i] = add(half, vel);
    s.visc[i] = viscosity;
    s.has[i] = 1;
    const V3 uu = s.u[i];
    const double usq = norm2(uu);
    for (int j = 0; j < Q; ++j) {
        const double vu = dot(uu, cvec(j));
        const double fe = W[j] * density * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
        s.f[i * Q + j] = fe;
        s.fs[i * Q + j] = fe;
    }
}

// ---- initialisation -----------------------------------------------------------------

bool buildLattice(hbo_sim& s, const hb_elements* e, const hb_objects* o) {
    const hb_params& P = s.P;
    const int X = s.X, Y = s.Y, Z = s.Z;
    const size_t N = s.N;
    s.type.assign(N, 0);
    s.inside.assign(N, 0);
    s.has.assign(N, 0);
    s.solid.assign(N, 0);
    s.nb.assign(N * Q, 0);
    s.f.assign(N * Q, 0.0);
    s.fs.assign(N * Q, 0.0);
    s.n.assign(N, 0.0);
    s.mass.assign(N, 0.0);
    s.newMass.assign(N, 0.0);
    s.visc.assign(N, 1.0);
    s.u.assign(N, v3(0, 0, 0));
    s.hf.assign(N, v3(0, 0, 0));
    const int64_t ne[Q] = {0, 1, -1, X, -X, (int64_t)X * Y, -(int64_t)X * Y, 1 + X, -1 - X, -1 + X,
                           1 - X, X + (int64_t)X * Y, -X - (int64_t)X * Y, -X + (int64_t)X * Y,
                           X - (int64_t)X * Y, (int64_t)X * Y + 1, -(int64_t)X * Y - 1,
                           -(int64_t)X * Y + 1, (int64_t)X * Y - 1};  // LB.cpp:57-81
    for (size_t i = 0; i < N; ++i)
        for (int j = 1; j < Q; ++j) s.nb[i * Q + j] = (uint32_t)((int64_t)i + ne[j]);  // LB.cpp:379-387
    for (size_t i = 0; i < N; ++i) s.nb[i * Q] = (uint32_t)i;
    // boundary layers: x, y, z in turn, a wall already set stays (LB.cpp:393-432)
    auto setb = [&](size_t i, int code) {
        s.type[i] = (uint8_t)code;
        for (int j = 0; j < Q; ++j) s.nb[i * Q + j] = (uint32_t)i;
    };
    for (size_t i = 0; i < N; ++i) {
        const int x = s.gx(i), y = s.gy(i), z = s.gz(i);
        if (x == 0 && !s.isWall(i)) setb(i, P.boundary[0]);
        else if (x == X - 1 && !s.isWall(i)) setb(i, P.boundary[1]);
        if (y == 0 && !s.isWall(i)) setb(i, P.boundary[2]);
        else if (y == Y - 1 && !s.isWall(i)) setb(i, P.boundary[3]);
        if (z == 0 && !s.isWall(i)) setb(i, P.boundary[4]);
        else if (z == Z - 1 && !s.isWall(i)) setb(i, P.boundary[5]);
    }
    // periodic remap of fluid nodes' links (LB.cpp:437-472)
    const int64_t dom[3] = {X - 2, (int64_t)X * Y - 2 * X, (int64_t)X * Y * Z - 2 * (int64_t)X * Y};
    for (size_t i = 0; i < N; ++i) {
        if (s.type[i] != 0) continue;
        const uint32_t* d = &s.nb[i * Q];
        const bool p1 = s.type[d[1]] == 4, p2 = s.type[d[2]] == 4, p3 = s.type[d[3]] == 4,
                   p4 = s.type[d[4]] == 4, p5 = s.type[d[5]] == 4, p6 = s.type[d[6]] == 4;
        int64_t pbc[Q] = {0};
        for (int j = 1; j < Q; ++j) {
            if (p1 && CX[j] > 0) pbc[j] -= dom[0];
            if (p2 && CX[j] < 0) pbc[j] += dom[0];
            if (p3 && CY[j] > 0) pbc[j] -= dom[1];
            if (p4 && CY[j] < 0) pbc[j] += dom[1];
            if (p5 && CZ[j] > 0) pbc[j] -= dom[2];
            if (p6 && CZ[j] < 0) pbc[j] += dom[2];
        }
        for (int j = 1; j < Q; ++j) s.nb[i * Q + j] = (uint32_t)((int64_t)s.nb[i * Q + j] + pbc[j]);
    }
    // particle flags: last particle in list order containing the node wins (LB.cpp:475-495)
    if (e) {  // every particle, ghosts included (LB.cpp:475-495)
        for (size_t p = 0; p < s.parts.size(); ++p) {
            const V3 c = s.parts[p].x0;
            const double r = s.parts[p].r;
            const int x0 = std::max(0, (int)std::floor(c.x - r) - 1), x1 = std::min(X - 1, (int)std::ceil(c.x + r) + 1);
            const int y0 = std::max(0, (int)std::floor(c.y - r) - 1), y1 = std::min(Y - 1, (int)std::ceil(c.y + r) + 1);
            const int z0 = std::max(0, (int)std::floor(c.z - r) - 1), z1 = std::min(Z - 1, (int)std::ceil(c.z + r) + 1);
            for (int z = z0; z <= z1; ++z)
                for (int y = y0; y <= y1; ++y)
                    for (int x = x0; x <= x1; ++x) {
                        const size_t i = s.idx(x, y, z);
                        if (!s.isActive(i)) continue;
                        if (norm2(sub(s.pos(i), c)) < r * r) {  // insideSphere, vector.cpp:153-158
                            s.inside[i] = 1;
                            s.solid[i] = (uint32_t)p;
                        }
                    }
        }
    }
    // walls from the boundary codes (DEM.cpp:435-633) mark their planes (LB.cpp:497-533)
    for (size_t w = 0; w < s.walls.size(); ++w) {
        const Wall& W0 = s.walls[w];
        for (size_t i = 0; i < N; ++i) {
            if (dot(W0.n, sub(s.pos(i), W0.p)) < 0.0) {  // insidePlane, vector.cpp:172-175
                s.solid[i] = (uint32_t)w;
                s.type[i] = W0.slip ? (W0.moving ? 6 : 5) : (W0.moving ? 8 : 7);
            }
        }
    }
    // cylinders: nodes outside become curved walls (LB.cpp:552-586)
    for (size_t ic = 0; ic < s.cyl.size(); ++ic)
        for (size_t i = 0; i < N; ++i)
            if (!insideCylinder(s.pos(i), s.cyl[ic].p1, s.cyl[ic].naxes, s.cyl[ic].R)) s.type[i] = 9;
    // objects become static wall nodes (LB.cpp:535-550)
    for (size_t io = 0; io < s.obj.size(); ++io) {
        const Object& ob = s.obj[io];
        for (size_t i = 0; i < N; ++i) {
            if (norm2(sub(s.pos(i), ob.x0)) < ob.r * ob.r) {
                s.solid[i] = (uint32_t)io;
                s.type[i] = 7;
            }
        }
    }
    // curve::delta of every curved node toward its non-wall neighbours, from the first
    // cylinder (LB.cpp:589-603, cylinder::segmentIntercept utils.cpp:177-224)
    if (!s.cyl.empty()) {
        s.delta.assign(N * Q, 0.0);
        for (size_t i = 0; i < N; ++i) {
            if (s.type[i] != 9) continue;
            for (int j = 1; j < Q; ++j) {
                const uint32_t l = s.nb[i * Q + j];
                if (s.isWall(l)) continue;
                s.delta[i * Q + j] = 1.0 - segmentIntercept(s.cyl[0], s.pos(i), cvec(j));
            }
        }
    }
    // dam-break column (gas outside x < gx*X, z < gz*Z), then the generic interface
    // loops of initializeInterface (LB.cpp:787-814)
    if (P.gas_box[0] > 0.0 || P.gas_box[1] > 0.0) {
        const double xl = P.gas_box[0] * X, zl = P.gas_box[1] * Z;
        for (size_t i = 0; i < N; ++i)
            if (s.type[i] == 0 && (s.gx(i) >= xl || s.gz(i) >= zl)) s.type[i] = 2;
    }
    for (size_t i = 0; i < N; ++i) {
        if (s.type[i] != 0) continue;
        for (int j = 1; j < Q; ++j)
            if (s.type[s.nb[i * Q + j]] == 2) s.type[i] = 3;
    }
    for (size_t i = 0; i < N; ++i) {
        if (s.type[i] != 3) continue;
        bool close = false;
        for (int j = 1; j < Q; ++j)
            if (s.type[s.nb[i * Q + j]] == 0) { close = true; break; }
        if (!close) s.type[i] = 2;
    }
    // lists (LB.cpp:817-876)
    for (size_t i = 0; i < N; ++i) {
        if (s.type[i] == 0) s.fluidNodes.push_back((uint32_t)i);
        else if (s.type[i] == 3) s.interfaceNodes.push_back((uint32_t)i);
        if (s.inside[i]) s.particleNodes.push_back((uint32_t)i);
    }
    // hydrostatic variables (LB.cpp:909-944)
    unsigned mx = 0, my = 0, mz = 0;
    for (size_t i = 0; i < N; ++i)
        if (s.isActive(i)) {
            mx = std::max(mx, (unsigned)s.gx(i));
            my = std::max(my, (unsigned)s.gy(i));
            mz = std::max(mz, (unsigned)s.gz(i));
        }
    const V3 maxP = v3(mx, my, mz);
    const V3 iv = v3(P.init_velocity[0], P.init_velocity[1], P.init_velocity[2]);
    for (size_t i = 0; i < N; ++i) {
        if (s.type[i] == 0) {
            const V3 dh = sub(s.pos(i), maxP);
            nodeInit(s, i, 1.0 + 3.0 * 1.0 * 1.0 * 1.0 * dot(dh, s.lbF), iv, 1.0, P.init_visc, s.lbF);
        } else if (s.type[i] == 3) {
            nodeInit(s, i, 1.0, iv, 0.5 * 1.0, P.init_visc, s.lbF);
        }
    }
    // wall nodes next to non-wall nodes (LB.cpp:946-996)
    for (size_t i = 0; i < N; ++i) {
        if (s.isWall(i)) continue;
        for (int j = 0; j < Q; ++j) {
            const uint32_t l = s.nb[i * Q + j];
            if (s.has[l]) continue;
            if (s.type[l] == 7 || s.type[l] == 5) {
                nodeInit(s, l, 1.0, v3(0, 0, 0), 0.0, 0.0, v3(0, 0, 0));
            } else if (s.type[l] == 8 || s.type[l] == 6 || s.type[l] == 9) {
                // the wall whose plane holds the node, else the cylinder it is outside of,
                // else the object it is inside of (LB.cpp:969-990)
                V3 vel = v3(0, 0, 0);
                const uint32_t si = s.solid[l];
                if (si < s.walls.size() && dot(s.walls[si].n, sub(s.pos(l), s.walls[si].p)) < 0.0)
                    vel = s.walls[si].speed(s.pos(l));
                else if (si < s.cyl.size() && !insideCylinder(s.pos(l), s.cyl[si].p1, s.cyl[si].naxes, s.cyl[si].R))
                    vel = cylinderSpeed(s.cyl[si], s.pos(l));
                else if (si < s.obj.size() && norm2(sub(s.pos(l), s.obj[si].x0)) < s.obj[si].r * s.obj[si].r)
                    vel = s.obj[si].x1;
                nodeInit(s, l, 1.0, vel, 0.0, 0.0, v3(0, 0, 0));
            }
        }
    }
    s.activeNodes.clear();
    s.activeNodes.insert(s.activeNodes.end(), s.fluidNodes.begin(), s.fluidNodes.end());
    s.activeNodes.insert(s.activeNodes.end(), s.interfaceNodes.begin(), s.interfaceNodes.end());
    std::sort(s.activeNodes.begin(), s.activeNodes.end());
    s.totalMass = 0.0;  // LB.cpp:204-218
    for (size_t i = 0; i < N; ++i)
        if (s.isActive(i) && !s.inside[i]) s.totalMass += s.mass[i];
    (void)o;
    return true;
}

void buildWalls(hbo_sim& s) {  // DEM.cpp:435-633
    const hb_params& P = s.P;
    const V3 ps[6] = {v3(0.5, 0, 0), v3(s.X - 1.5, 0, 0), v3(0, 0.5, 0),
                      v3(0, s.Y - 1.5, 0), v3(0, 0, 0.5), v3(0, 0, s.Z - 1.5)};
    const V3 ns[6] = {v3(1, 0, 0), v3(-1, 0, 0), v3(0, 1, 0), v3(0, -1, 0), v3(0, 0, 1), v3(0, 0, -1)};
    for (int k = 0; k < 6; ++k) {
        const int b = P.boundary[k];
        if (b >= 5 && b <= 8) {
            Wall w;
            w.p = ps[k];
            w.n = ns[k];
            w.moving = (b == 8 || b == 6);
            w.slip = (b == 5 || b == 6);
            w.vel = v3(0, 0, 0);
            w.omega = v3(0, 0, 0);
            w.rot = (k == 2) ? v3(0.0, 0.5 + 0.4, 1.260) : v3(0, 0, 0);
            w.fhydro = v3(0, 0, 0);
            w.fparticle = v3(0, 0, 0);
            s.walls.push_back(w);
        }
    }
}

void initNeighborParameters(hbo_sim& s) {  // DEM.cpp:1270-1312
    double maxRad = 0.0;
    for (auto& e : s.el) maxRad = std::max(maxRad, e.radius);
    const double demSize[3] = {(double)s.X, (double)s.Y, (double)s.Z};
    for (int k = 0; k < 3; ++k) {
        s.cellWidth[k] = s.el.empty() ? demSize[k] : std::min(maxRad * 5.0, demSize[k]);
        s.nCells[k] = (unsigned)(int)std::ceil(demSize[k] / s.cellWidth[k]);
        s.cellWidth[k] = demSize[k] / double(s.nCells[k]);
        s.nCells[k] += 2;
    }
    s.nebrRange = std::max(maxRad * 3.0, 0.5 * std::min(s.cellWidth[0], std::min(s.cellWidth[1], s.cellWidth[2])));
    s.maxDisp = 0.5 * s.nebrRange;
}

// particle::updatePredicted / updateCorrected (elmt.cpp:261-290) for the standard
// particles, particle::ghostUpdate (elmt.cpp:292-299) for the ghosts (DEM.cpp:1184-1230)
void updateParticles(hbo_sim& s, bool predicted) {
    for (unsigned p = 0; p < s.stdParticles; ++p) {
        Part& q = s.parts[p];
        const Elmt& e = s.el[q.cluster];
        q.x0 = predicted ? e.xp0 : e.x0;
        q.radiusVec = v3(0, 0, 0);
        q.x1 = predicted ? e.xp1 : e.x1;
        if (e.size > 1) {
            q.x0 = add(q.x0, mul(q.r, project(prototype(e.size, q.proto), predicted ? e.qp0 : e.q0)));
            q.radiusVec = sub(q.x0, predicted ? e.xp0 : e.x0);
            q.x1 = add(q.x1, cross(predicted ? e.wpGlobal : e.wGlobal, q.radiusVec));
        }
    }
    for (size_t g = 0; g < s.ghosts.size(); ++g) {
        Part& q = s.parts[s.stdParticles + g];
        const Part& o = s.parts[s.ghosts[g].index];
        q.x0 = add(o.x0, s.ghosts[g].vec);
        q.radiusVec = o.radiusVec;
        q.x1 = o.x1;
    }
}

void pbcShift(hbo_sim& s) {  // DEM.cpp:1554-1584 (elmt::translate moves x0 and xp0)
    for (const Pbc& b : s.pbcs)
        for (auto& e : s.el) {
            const double ld = b.dist1(e.x0), rd = b.dist2(e.x0);
            if (ld < 0.0) { e.x0 = add(e.x0, b.v); e.xp0 = add(e.xp0, b.v); }
            if (rd < 0.0) { const V3 mv = mul(-1.0, b.v); e.x0 = add(e.x0, mv); e.xp0 = add(e.xp0, mv); }
        }
}

void createGhosts(hbo_sim& s) {  // DEM.cpp:1586-1664
    s.ghosts.clear();
    for (const Pbc& b : s.pbcs)
        for (size_t n = 0; n < s.el.size(); ++n)
            for (unsigned j = 0; j < (unsigned)s.el[n].size; ++j) {
                const unsigned p = s.comps[n][j];
                if (b.dist1(s.parts[p].x0) < s.nebrRange) s.ghosts.push_back(Ghost{p, b.v});
                else if (b.dist2(s.parts[p].x0) < s.nebrRange) s.ghosts.push_back(Ghost{p, mul(-1.0, b.v)});
            }
    const size_t ns = s.ghosts.size();
    for (size_t g1 = 0; g1 < ns; ++g1)
        for (size_t g2 = g1 + 1; g2 < ns; ++g2)
            if (s.ghosts[g1].index == s.ghosts[g2].index)
                s.ghosts.push_back(Ghost{s.ghosts[g1].index, add(s.ghosts[g1].vec, s.ghosts[g2].vec)});
    s.parts.resize(s.stdParticles);
    for (size_t n = 0; n < s.el.size(); ++n) s.comps[n].resize(s.el[n].size);
    for (size_t g = 0; g < s.ghosts.size(); ++g) {
        Part q = s.parts[s.ghosts[g].index];
        s.comps[q.cluster].push_back(s.stdParticles + (unsigned)g);
        s.parts.push_back(q);
    }
}

void evalNeighborTable(hbo_sim& s) {  // DEM.cpp:1326-1513 (cell table, half-shell sweep)
    static const int shift[14][3] = {{0, 0, 0},  {1, 0, 0},  {1, 1, 0},  {0, 1, 0},  {-1, 1, 0},
                                     {0, 0, 1},  {1, 0, 1},  {1, 1, 1},  {0, 1, 1},  {-1, 1, 1},
                                     {-1, 0, 1}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1}};
    if (!s.pbcs.empty()) {  // DEM.cpp:1395-1411
        s.ghosts.clear();
        s.parts.resize(s.stdParticles);
        for (size_t n = 0; n < s.el.size(); ++n) s.comps[n].resize(s.el[n].size);
        pbcShift(s);
        updateParticles(s, false);
        createGhosts(s);
        updateParticles(s, false);
        s.newNeighborList = true;
    }
    const unsigned P = (unsigned)s.parts.size();
    const unsigned nc = s.nCells[0] * s.nCells[1] * s.nCells[2];
    s.cellTable.assign(P + nc, -1);
    s.tableCell.assign(P, 0);
    for (unsigned n = 0; n < P; ++n) {
        const V3 x = s.parts[n].x0;  // linearizePosition, vector.cpp:147-149
        const int c = (int)(std::floor(x.x / s.cellWidth[0]) + 1 +
                            s.nCells[0] * (std::floor(x.y / s.cellWidth[1]) + 1 +
                                           (s.nCells[1] * (std::floor(x.z / s.cellWidth[2])) + 1))) +
                      (int)P;
        if (c >= (int)(P + nc) || c < 0) {
            g_err = "particle outside the DEM box";
            continue;
        }
        s.tableCell[n] = c;
        s.cellTable[n] = s.cellTable[c];
        s.cellTable[c] = (int)n;
    }
    const double r2 = s.nebrRange * s.nebrRange;
    s.neighborTable.clear();
    unsigned i0[3];
    for (i0[0] = 0; i0[0] < s.nCells[0]; ++i0[0])
        for (i0[1] = 0; i0[1] < s.nCells[1]; ++i0[1])
            for (i0[2] = 0; i0[2] < s.nCells[2]; ++i0[2])
                for (int sh = 0; sh < 14; ++sh) {
                    unsigned i1[3];
                    for (int k = 0; k < 3; ++k) {
                        i1[k] = i0[k] + (unsigned)shift[sh][k];
                        if (i1[k] == s.nCells[k]) i1[k] = 0;
                    }
                    const unsigned cell0 = (i0[2] * s.nCells[1] + i0[1]) * s.nCells[0] + i0[0] + P;
                    const unsigned cell1 = (i1[2] * s.nCells[1] + i1[1]) * s.nCells[0] + i1[0] + P;
                    if (cell1 >= s.cellTable.size()) continue;  // never reached for in-box particles
                    int n0 = s.cellTable[cell0];
                    while (n0 > -1) {
                        int n1 = s.cellTable[cell1];
                        while (n1 > -1) {
                            if (cell0 != cell1 || n1 < n0) {
                                if (s.parts[n0].cluster != s.parts[n1].cluster) {
                                    const V3 r10 = sub(s.parts[n1].x0, s.parts[n0].x0);
                                    if (norm2(r10) < r2) {
                                        s.neighborTable.push_back((uint32_t)n0);
                                        s.neighborTable.push_back((uint32_t)n1);
                                    }
                                }
                            }
                            n1 = s.cellTable[n1];
                        }
                        n0 = s.cellTable[n0];
                    }
                }
    const unsigned Ps = s.stdParticles;
    s.nearWallTable.clear();  // DEM.cpp:1496-1513: first wall in range only
    for (unsigned n = 0; n < Ps; ++n)
        for (size_t w = 0; w < s.walls.size(); ++w)
            if (s.walls[w].dist(s.parts[n].x0) < s.nebrRange) {
                s.nearWallTable.push_back(n);
                s.nearWallTable.push_back((uint32_t)w);
                break;
            }
    s.nearObjectTable.clear();  // DEM.cpp:1515-1533
    for (unsigned n = 0; n < Ps; ++n)
        for (size_t o = 0; o < s.obj.size(); ++o)
            if (norm2(sub(s.parts[n].x0, s.obj[o].x0)) < r2) {
                s.nearObjectTable.push_back(n);
                s.nearObjectTable.push_back((uint32_t)o);
            }
    s.nearCylinderTable.clear();  // DEM.cpp:1535-1550: first cylinder in range only
    for (unsigned n = 0; n < Ps; ++n)
        for (size_t c = 0; c < s.cyl.size(); ++c)
            if (cylinderDist(s.cyl[c], s.parts[n].x0) < s.nebrRange) {
                s.nearCylinderTable.push_back(n);
                s.nearCylinderTable.push_back((uint32_t)c);
                break;
            }
}

// ---- DEM ----------------------------------------------------------------------------

double normalContact(const hbo_sim& s, double overlap, double vn, double effRad, double effMass) {
    // DEM.cpp:2138-2174
    if (s.P.contact_model == HB_HERTZIAN) {
        const double kn = s.knConst * std::sqrt(effRad) * std::sqrt(overlap);
        const double gn = 2.0 * s.dampCoeff * std::sqrt(kn * effMass);
        return std::max(kn * overlap + (-gn * vn), 0.0);
    }
    const double el = s.P.linear_stiff * overlap;
    const double gn = 2.0 * s.dampCoeff * std::sqrt(s.P.linear_stiff * effMass);
    return std::max(el + (-gn * vn), 0.0);
}

double tangentialContact(const hbo_sim& s, double vt, double fn, double effRad, double effMass,
                         double friction) {  // DEM.cpp:2176-2222
    double ks;
    if (s.P.contact_model == HB_HERTZIAN) ks = s.ksConst * std::sqrt(effRad) * std::pow(std::abs(fn), 1.0 / 3.0);
    else ks = s.P.linear_stiff;
    const double fsMax = friction * fn;
    const double gs = 2.0 * s.P.visc_tang * std::sqrt(effMass * ks);
    return std::min(gs * vt, fsMax);
}

// the element sides take forces only from standard particles (DEM.cpp:1845-1858,
// 1879-1888); the normal force has a moment on multi-sphere elements
void particleParticleCollision(hbo_sim& s, unsigned i, unsigned j, V3 vd) {  // DEM.cpp:1801-1900
    const Part& pI = s.parts[i];
    const Part& pJ = s.parts[j];
    Elmt& A = s.el[pI.cluster];
    Elmt& B = s.el[pJ.cluster];
    const double radI = pI.r, radJ = pJ.r;
    const double distance = norm(vd);
    const double overlap = radI + radJ - distance;
    const V3 relVel = sub(pJ.x1, pI.x1);
    const V3 en = divs(vd, distance);
    const double normRelVel = dot(relVel, en);
    const V3 normalRelVel = mul(normRelVel, en);
    const double effMass = A.m * B.m / (A.m + B.m);
    const double effRad = radI * radJ / (radI + radJ);
    const double fn = normalContact(s, overlap, normRelVel, effRad, effMass);
    const V3 normalForce = mul(fn, en);
    const V3 vecRadI = mul(radI, en);
    const V3 vecRadJ = mul(-radJ, en);
    const V3 cI = add(vecRadI, pI.radiusVec), cJ = add(vecRadJ, pJ.radiusVec);
    const bool stdI = i < s.stdParticles, stdJ = j < s.stdParticles;
    if (stdI) {
        A.FParticle = sub(A.FParticle, normalForce);
        if (A.size > 1) A.MParticle = sub(A.MParticle, cross(cI, normalForce));
    }
    if (stdJ) {
        B.FParticle = add(B.FParticle, normalForce);
        if (B.size > 1) B.MParticle = add(B.MParticle, cross(cJ, normalForce));
    }
    const V3 relVelContact = add(sub(relVel, cross(A.wpGlobal, vecRadI)), cross(B.wpGlobal, vecRadJ));
    const V3 tang = sub(relVelContact, normalRelVel);
    const double nt = norm(tang);
    if (nt != 0.0) {
        const double ft = tangentialContact(s, nt, fn, effRad, effMass, s.P.friction_part);
        const V3 et = divs(tang, nt);
        const V3 tf = mul(ft, et);
        if (stdI) {
            A.MParticle = add(A.MParticle, cross(cI, tf));
            A.FParticle = add(A.FParticle, tf);
        }
        if (stdJ) {
            B.MParticle = sub(B.MParticle, cross(cJ, tf));
            B.FParticle = sub(B.FParticle, tf);
        }
    }
}

void wallParticleCollision(hbo_sim& s, Wall& w, unsigned j, double overlap) {  // DEM.cpp:1902-1982
    const Part& pJ = s.parts[j];
    Elmt& B = s.el[pJ.cluster];
    const double radJ = pJ.r;
    const V3 en = w.n;
    const V3 relVel = sub(pJ.x1, w.speed(pJ.x0));
    const double vn = dot(relVel, en);
    const V3 nrv = mul(vn, en);
    const double fn = normalContact(s, 2.0 * overlap, vn, radJ, B.m);
    const V3 nf = mul(fn, en);
    const V3 vecRadJ = mul(-radJ, en);
    V3 cJ = vecRadJ;
    if (B.size > 1) cJ = add(cJ, sub(pJ.x0, B.xp0));
    B.FWall = add(B.FWall, nf);
    w.fparticle = sub(w.fparticle, nf);
    if (B.size > 1) B.MWall = add(B.MWall, cross(cJ, nf));
    const V3 rvc = add(relVel, cross(B.wpGlobal, vecRadJ));
    const V3 tang = sub(rvc, nrv);
    const double nt = norm(tang);
    if (nt != 0.0) {
        const double ft = tangentialContact(s, nt, fn, radJ, B.m, s.P.friction_wall);
        const V3 et = divs(tang, norm(tang));
        const V3 tf = mul(ft, et);
        B.MWall = sub(B.MWall, cross(cJ, tf));
        B.FWall = sub(B.FWall, tf);
        w.fparticle = add(w.fparticle, tf);
    }
}

void cylinderParticleCollision(hbo_sim& s, const Cyl& c, unsigned j, double overlap) {  // DEM.cpp:1984-2058
    const Part& pJ = s.parts[j];
    Elmt& B = s.el[pJ.cluster];
    const double radJ = pJ.r;
    const V3 vd = cylinderVecDist(c, pJ.x0);
    const V3 cp = sub(pJ.x0, vd);
    const V3 en = divs(vd, radJ - overlap);
    const V3 relVel = sub(pJ.x1, cylinderSpeed(c, cp));
    const double vn = dot(relVel, en);
    const V3 nrv = mul(vn, en);
    const double fn = normalContact(s, 2.0 * overlap, vn, radJ, B.m);
    const V3 nf = mul(fn, en);
    const V3 vecRadJ = mul(-radJ, en);
    const V3 cJ = add(vecRadJ, sub(pJ.x0, B.xp0));
    B.FWall = add(B.FWall, nf);
    if (B.size > 1) B.MWall = add(B.MWall, cross(cJ, nf));
    const V3 rvc = add(relVel, cross(B.wpGlobal, vecRadJ));
    const V3 tang = sub(rvc, nrv);
    const double nt = norm(tang);
    if (nt != 0.0) {
        const double ft = tangentialContact(s, nt, fn, radJ, B.m, s.P.friction_wall);
        const V3 et = divs(tang, norm(tang));
        const V3 tf = mul(ft, et);
        B.MWall = sub(B.MWall, cross(cJ, tf));
        B.FWall = sub(B.FWall, tf);
    }
}

void objectParticleCollision(hbo_sim& s, Object& o, unsigned j, V3 vd) {  // DEM.cpp:2060-2136
    const Part& pJ = s.parts[j];
    Elmt& B = s.el[pJ.cluster];
    const double radJ = pJ.r;
    const double distance = norm(vd);
    const double overlap = radJ + o.r - distance;
    const V3 en = mul(1.0 / distance, vd);
    const V3 relVel = sub(pJ.x1, o.x1);
    const double vn = dot(relVel, en);
    const V3 nrv = mul(vn, en);
    const double fn = normalContact(s, 2.0 * overlap, vn, radJ, B.m);
    const V3 nf = mul(fn, en);
    const V3 vecRadJ = mul(-radJ, en);
    const V3 cJ = add(vecRadJ, sub(pJ.x0, B.xp0));
    B.FWall = add(B.FWall, nf);
    o.fparticle = sub(o.fparticle, nf);
    if (B.size > 1) B.MWall = add(B.MWall, cross(cJ, nf));
    const V3 rvc = add(relVel, cross(B.wpGlobal, vecRadJ));
    const V3 tang = sub(rvc, nrv);
    const double nt = norm(tang);
    if (nt != 0.0) {
        const double ft = tangentialContact(s, nt, fn, radJ, B.m, s.P.friction_part);
        const V3 et = divs(tang, norm(tang));
        const V3 tf = mul(ft, et);
        B.MWall = sub(B.MWall, cross(cJ, tf));
        B.FWall = sub(B.FWall, tf);
        o.fparticle = add(o.fparticle, tf);
    }
}

void demSubstep(hbo_sim& s) {  // DEM.cpp:336-374
    s.demTime += s.deltat;
    // evalMaxDisp + rebuild trigger captured at the first call (DEM.cpp:334, 1314-1324)
    if (!s.triggerSet) {
        s.trigger = 0.25 * s.nebrRange;
        s.triggerSet = true;
    }
    double maxVel = 0.0;
    for (auto& e : s.el)
        if (norm2(e.x1) > maxVel) maxVel = norm2(e.x1);
    maxVel = std::sqrt(maxVel);
    s.maxDisp += maxVel * s.deltat;
    if (s.maxDisp > s.trigger) {
        s.maxDisp = 0.0;
        evalNeighborTable(s);
    }
    // predictor (DEM.cpp:1067-1080, elmt.cpp:139-177)
    const double dt = s.deltat;
    const double c[5] = {dt, dt * dt / 2.0, dt * dt * dt / 6.0, dt * dt * dt * dt / 24.0,
                         dt * dt * dt * dt * dt / 120.0};
    for (auto& e : s.el) {
        e.xp0 = add(add(add(add(add(e.x0, mul(c[0], e.x1)), mul(c[1], e.x2)), mul(c[2], e.x3)), mul(c[3], e.x4)), mul(c[4], e.x5));
        e.xp1 = add(add(add(add(e.x1, mul(c[0], e.x2)), mul(c[1], e.x3)), mul(c[2], e.x4)), mul(c[3], e.x5));
        e.xp2 = add(add(add(e.x2, mul(c[0], e.x3)), mul(c[1], e.x4)), mul(c[2], e.x5));
        e.xp3 = add(add(e.x3, mul(c[0], e.x4)), mul(c[1], e.x5));
        e.xp4 = add(e.x4, mul(c[0], e.x5));
        e.xp5 = e.x5;
        e.qp0 = qadd(qadd(qadd(qadd(qadd(e.q0, qscale(e.q1, c[0])), qscale(e.q2, c[1])), qscale(e.q3, c[2])), qscale(e.q4, c[3])), qscale(e.q5, c[4]));
        e.qp1 = qadd(qadd(qadd(qadd(e.q1, qscale(e.q2, c[0])), qscale(e.q3, c[1])), qscale(e.q4, c[2])), qscale(e.q5, c[3]));
        e.qp2 = qadd(qadd(qadd(e.q2, qscale(e.q3, c[0])), qscale(e.q4, c[1])), qscale(e.q5, c[2]));
        e.qp3 = qadd(qadd(e.q3, qscale(e.q4, c[0])), qscale(e.q5, c[1]));
        e.qp4 = qadd(e.q4, qscale(e.q5, c[0]));
        e.qp5 = e.q5;
        qnormalize(e.qp0);
        e.wp0 = add(add(add(add(add(e.w0, mul(c[0], e.w1)), mul(c[1], e.w2)), mul(c[2], e.w3)), mul(c[3], e.w4)), mul(c[4], e.w5));
        e.wp1 = add(add(add(add(e.w1, mul(c[0], e.w2)), mul(c[1], e.w3)), mul(c[2], e.w4)), mul(c[3], e.w5));
        e.wp2 = add(add(add(e.w2, mul(c[0], e.w3)), mul(c[1], e.w4)), mul(c[2], e.w5));
        e.wp3 = add(add(e.w3, mul(c[0], e.w4)), mul(c[1], e.w5));
        e.wp4 = add(e.w4, mul(c[0], e.w5));
        e.wp5 = e.w5;
        e.wpGlobal = e.wp0;
        e.wpLocal = project(e.wpGlobal, qadj(e.qp0));
    }
    updateParticles(s, true);
    // forces (DEM.cpp:1114-1182)
    for (auto& e : s.el) {
        e.FParticle = e.FWall = e.MParticle = e.MWall = v3(0, 0, 0);
    }
    for (auto& w : s.walls) w.fparticle = v3(0, 0, 0);
    for (auto& o : s.obj) o.fparticle = v3(0, 0, 0);
    for (size_t k = 0; k < s.neighborTable.size(); k += 2) {  // DEM.cpp:1668-1690
        const unsigned i = s.neighborTable[k], j = s.neighborTable[k + 1];
        const double sig = s.parts[i].r + s.parts[j].r;
        const V3 vd = sub(s.parts[j].x0, s.parts[i].x0);
        if (norm2(vd) < sig * sig) particleParticleCollision(s, i, j, vd);
    }
    for (size_t k = 0; k < s.nearWallTable.size(); k += 2) {  // DEM.cpp:1692-1717
        const unsigned j = s.nearWallTable[k];
        Wall& w = s.walls[s.nearWallTable[k + 1]];
        const double overlap = s.parts[j].r - w.dist(s.parts[j].x0);
        if (overlap > 0.0) wallParticleCollision(s, w, j, overlap);
    }
    for (size_t k = 0; k < s.nearObjectTable.size(); k += 2) {  // DEM.cpp:1747-1770
        const unsigned j = s.nearObjectTable[k];
        Object& o = s.obj[s.nearObjectTable[k + 1]];
        const V3 vd = sub(s.parts[j].x0, o.x0);
        const double overlap = s.parts[j].r + o.r - norm(vd);
        if (overlap > 0.0) objectParticleCollision(s, o, j, vd);
    }
    for (size_t k = 0; k < s.nearCylinderTable.size(); k += 2) {  // DEM.cpp:1719-1746
        const unsigned j = s.nearCylinderTable[k];
        const Cyl& c = s.cyl[s.nearCylinderTable[k + 1]];
        const double overlap = s.parts[j].r - cylinderDist(c, s.parts[j].x0);
        if (overlap > 0.0) cylinderParticleCollision(s, c, j, overlap);
    }
    const double nv = s.P.num_visc;
    for (auto& e : s.el) {
        const V3 FVisc = mul(-6.0 * M_PI * nv * e.radius, e.xp1);
        const V3 MVisc = mul(-8.0 * M_PI * nv * e.radius * e.radius * e.radius, e.wpGlobal);
        e.x2 = add(divs(add(add(add(FVisc, e.FHydro), e.FParticle), e.FWall), e.m), s.demF);
        const V3 moment = add(add(add(MVisc, e.MHydro), e.MParticle), e.MWall);
        const V3 mBf = project(moment, qadj(e.qp0));
        const V3 waBf = newtonAcc(mBf, e.I, e.wpLocal);
        e.w1 = project(waBf, e.qp0);
        if (e.size > 1) {  // quatAcc (vector.cpp:500-504), DEM.cpp:1176-1179
            const double n2 = e.qp1.q0 * e.qp1.q0 + e.qp1.q1 * e.qp1.q1 + e.qp1.q2 * e.qp1.q2 + e.qp1.q3 * e.qp1.q3;
            e.q2 = qscale(qmul(e.qp0, Quat{-2.0 * n2, waBf.x, waBf.y, waBf.z}), 0.5);
        }
    }
    // corrector (DEM.cpp:1082-1112, elmt.cpp:179-254)
    const double g1[6] = {95.0 / 288.0, 1.0, 25.0 / 24.0, 35.0 / 72.0, 5.0 / 48.0, 1.0 / 120.0};
    const double g2[6] = {3.0 / 16.0, 251.0 / 360.0, 1.0, 11.0 / 18.0, 1.0 / 6.0, 1.0 / 60.0};
    const double c1o[6] = {g1[0] * c[0], g1[1] * c[0] / c[0], g1[2] * c[0] / c[1], g1[3] * c[0] / c[2],
                           g1[4] * c[0] / c[3], g1[5] * c[0] / c[4]};
    const double c2o[6] = {g2[0] * c[1], g2[1] * c[1] / c[0], g2[2] * c[1] / c[1], g2[3] * c[1] / c[2],
                           g2[4] * c[1] / c[3], g2[5] * c[1] / c[4]};
    for (auto& e : s.el) {
        const V3 x2c = sub(e.x2, e.xp2);
        e.x0 = add(e.xp0, mul(c2o[0], x2c));
        e.x1 = add(e.xp1, mul(c2o[1], x2c));
        e.x3 = add(e.xp3, mul(c2o[3], x2c));
        e.x4 = add(e.xp4, mul(c2o[4], x2c));
        e.x5 = add(e.xp5, mul(c2o[5], x2c));
        e.xp0 = e.x0; e.xp1 = e.x1; e.xp2 = e.x2; e.xp3 = e.x3; e.xp4 = e.x4; e.xp5 = e.x5;
        const V3 w1c = sub(e.w1, e.wp1);
        e.w0 = add(e.wp0, mul(c1o[0], w1c));
        e.w2 = add(e.wp2, mul(c1o[2], w1c));
        e.w3 = add(e.wp3, mul(c1o[3], w1c));
        e.w4 = add(e.wp4, mul(c1o[4], w1c));
        e.w5 = add(e.wp5, mul(c1o[5], w1c));
        e.wp0 = e.w0; e.wp1 = e.w1; e.wp2 = e.w2; e.wp3 = e.w3; e.wp4 = e.w4; e.wp5 = e.w5;
        const Quat q2c = qsub(e.q2, e.qp2);
        e.q0 = qadd(e.qp0, qscale(q2c, c2o[0]));
        e.q1 = qadd(e.qp1, qscale(q2c, c2o[1]));
        e.q3 = qadd(e.qp3, qscale(q2c, c2o[3]));
        e.q4 = qadd(e.qp4, qscale(q2c, c2o[4]));
        e.q5 = qadd(e.qp5, qscale(q2c, c2o[5]));
        qnormalize(e.q0);
        e.qp0 = e.q0; e.qp1 = e.q1; e.qp2 = e.q2; e.qp3 = e.q3; e.qp4 = e.q4; e.qp5 = e.q5;
        e.wGlobal = e.w0;
        e.wLocal = project(e.wGlobal, qadj(e.q0));
    }
    updateParticles(s, false);
}

// ---- LB -----------------------------------------------------------------------------

void cleanLists(hbo_sim& s) {  // LB.cpp:1000-1060
    auto sortu = [](std::vector<uint32_t>& v) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    };
    sortu(s.fluidNodes);
    sortu(s.interfaceNodes);
    sortu(s.particleNodes);
    s.activeNodes.clear();
    s.activeNodes.insert(s.activeNodes.end(), s.fluidNodes.begin(), s.fluidNodes.end());
    s.activeNodes.insert(s.activeNodes.end(), s.interfaceNodes.begin(), s.interfaceNodes.end());
    sortu(s.activeNodes);
    std::vector<uint32_t> keep;
    keep.reserve(s.activeNodes.size());
    for (size_t k = 0; k < s.activeNodes.size(); ++k)
        if (k == 0 || s.type[s.activeNodes[k]] != 2) keep.push_back(s.activeNodes[k]);
    s.activeNodes.swap(keep);
}

void reconstruct(hbo_sim& s, size_t i) {  // node::reconstruct, node.cpp:63-83
    const double* fi = &s.f[i * Q];
    double nn = 0.0;
    for (int j = 0; j < Q; ++j) nn += fi[j];
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int j = 0; j < Q; ++j) {
        ux += fi[j] * CX[j];
        uy += fi[j] * CY[j];
        uz += fi[j] * CZ[j];
    }
    s.n[i] = nn;
    s.u[i] = v3(ux / nn, uy / nn, uz / nn);
}

// Moving bounce-back coupling (not in the reference: its particle branch is commented out,
// LB.cpp:1247-1276, and is restated here with the moving-wall rule of LB.cpp:1321-1341).
// Velocity of the solid at node l inside a particle: the element's velocity plus its spin
// times the lever arm from the element centre, radius = pos - x0 + radiusVec.
V3 mbbVelocity(const hbo_sim& s, size_t l) {
    const Part& q = s.parts[s.solid[l]];
    const Elmt& e = s.el[q.cluster];
    const V3 radius = add(sub(s.pos(l), q.x0), q.radiusVec);
    return add(e.x1, cross(e.wGlobal, radius));
}

// Element force and torque of the moving bounce-back links (node::bounceBackForce,
// node.cpp:283-291): (2 (fs_j - w_j rho0) - BBi) c_j per fluid -> particle link, in
// node order then link order; fluidVolume counts the element's solid nodes.
void mbbForces(hbo_sim& s) {
    for (auto& e : s.el) {
        e.FHydro = v3(0, 0, 0);
        e.MHydro = v3(0, 0, 0);
        e.fluidVolume = 0.0;
    }
    for (size_t k = 0; k < s.activeNodes.size(); ++k) {
        const size_t i = s.activeNodes[k];
        if (s.inside[i]) {
            s.el[s.parts[s.solid[i]].cluster].fluidVolume += 1.0;
            continue;
        }
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[i * Q + j];
            if (!((s.type[l] == 0 || s.type[l] == 3) && s.inside[l])) continue;
            const Part& q = s.parts[s.solid[l]];
            Elmt& e = s.el[q.cluster];
            const V3 radius = add(sub(s.pos(l), q.x0), q.radiusVec);
            const double BBi = 6.0 * s.n[i] * W[j] * dot(add(e.x1, cross(e.wGlobal, radius)), cvec(j));
            const V3 BBforce = mul(2.0 * (s.fs[i * Q + j] - 1.0 * W[j]) - BBi, cvec(j));
            e.FHydro = add(e.FHydro, BBforce);
            e.MHydro = add(e.MHydro, cross(radius, BBforce));
        }
    }
}

void computeHydroForces(hbo_sim& s) {  // LB.cpp:1851-1919
    for (auto& e : s.el) {
        e.FHydro = v3(0, 0, 0);
        e.MHydro = v3(0, 0, 0);
        e.fluidVolume = 0.0;
    }
    for (size_t k = 0; k < s.activeNodes.size(); ++k) {
        const size_t i = s.activeNodes[k];
        s.hf[i] = v3(0, 0, 0);
        if (!s.inside[i]) continue;
        const Part& q = s.parts[s.solid[i]];
        Elmt& e = s.el[q.cluster];
        const V3 radius = add(sub(s.pos(i), q.x0), q.radiusVec);
        const V3 localVel = add(e.x1, cross(e.wGlobal, radius));
        const V3 diffVel = mul(s.mass[i] / s.n[i], sub(s.u[i], localVel));
        s.hf[i] = add(s.hf[i], mul(-1.0, diffVel));
        e.fluidVolume += s.mass[i];
        e.FHydro = add(e.FHydro, mul(1.0, diffVel));
        e.MHydro = add(e.MHydro, mul(1.0, cross(radius, diffVel)));
    }
}

void collideNode(hbo_sim& s, size_t i) {  // LB.cpp:1094-1111, node.cpp:85-184
    const hb_params& P = s.P;
    double* fi = &s.f[i * Q];
    const double nn = s.n[i];
    const V3 tf = add(s.lbF, s.hf[i]);
    s.u[i] = add(s.u[i], divs(mul(0.5 * 1.0, tf), nn));  // shiftVelocity
    const V3 uu = s.u[i];
    const double usq = norm2(uu);
    double feq[Q];
    for (int j = 0; j < Q; ++j) {
        const double vu = dot(uu, cvec(j));
        feq[j] = W[j] * nn * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
    }
    if (P.non_newtonian || P.turbulence) {  // computeShearRate, node.cpp:103-145
        const double minVisc = (MIN_TAU - 0.5) / 3 / 1.0, maxVisc = (MAX_TAU - 0.5) / 3 / 1.0;
        const double tau = 0.5 + 3.0 * s.visc[i] * 1.0;
        double g[9] = {0};
        for (int j = 0; j < Q; ++j) {
            const double d = fi[j] - feq[j];
            const double c3[3] = {(double)CX[j], (double)CY[j], (double)CZ[j]};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) g[a * 3 + b] += d * (c3[a] * c3[b]);
        }
        const double sc = 1.5 * 1.0 / (tau * nn);
        for (int k = 0; k < 9; ++k) g[k] *= sc;
        const double shear = std::sqrt(0.5 * (g[0] * g[0] + g[4] * g[4] + g[8] * g[8] +
                                              2.0 * (g[1] * g[3] + g[6] * g[2] + g[5] * g[7])));
        const double nuTurb = P.turbulence ? P.turb_const * shear : 0.0;
        const double nuApp = P.non_newtonian ? P.plastic_visc + P.yield_stress / (nn * 2.0 * shear) : s.visc[i];
        s.visc[i] = std::max(minVisc, std::min(maxVisc, nuApp + nuTurb));
    }
    const double visc = s.visc[i];
    if (P.collision == HB_TRT) {
        // TRT: symmetric part relaxed with 1/tau, antisymmetric with the magic-parameter rate
        const double tp = 0.5 + 3.0 * visc;
        const double tm = P.trt_magic / (tp - 0.5) + 0.5;
        const double wp = 1.0 / tp, wm = 1.0 / tm;
        double fn[Q];
        for (int j = 0; j < Q; ++j) {
            const int o = OPP[j];
            const double fp = 0.5 * (fi[j] + fi[o]), fm = 0.5 * (fi[j] - fi[o]);
            const double ep = 0.5 * (feq[j] + feq[o]), em = 0.5 * (feq[j] - feq[o]);
            fn[j] = fi[j] - wp * (fp - ep) - wm * (fm - em);
        }
        // Guo force split into symmetric / antisymmetric parts with (1 - w/2) factors
        const double ap = 1.0 - 0.5 * wp, am = 1.0 - 0.5 * wm;
        double Fi[Q];
        for (int j = 0; j < Q; ++j) {
            const V3 cj = cvec(j);
            const double vu = dot(uu, cj);
            const V3 fpv = add(mul(9.0 * vu, cj), mul(3.0, sub(cj, uu)));
            Fi[j] = W[j] * dot(fpv, tf);
        }
        for (int j = 0; j < Q; ++j) {
            const int o = OPP[j];
            fi[j] = fn[j] + ap * 0.5 * (Fi[j] + Fi[o]) + am * 0.5 * (Fi[j] - Fi[o]);
        }
        return;
    }
    const double omega = 1.0 / (0.5 + 3.0 * visc * 1.0);  // solveCollision
    for (int j = 0; j < Q; ++j) fi[j] += omega * (feq[j] - fi[j]);
    const double omegaf = 1.0 - 1.0 / (1.0 + 6.0 * visc * 1.0);  // addForce
    for (int j = 0; j < Q; ++j) {
        const V3 cj = cvec(j);
        const double vu = dot(uu, cj);
        const V3 vmu = sub(cj, uu);
        const V3 fp = add(mul(9.0 * vu, cj), mul(3.0, vmu));
        fi[j] += 1.0 * omegaf * W[j] * dot(fp, tf);
    }
}

bool streaming(hbo_sim& s) {  // LB.cpp:1144-1488
    for (auto& w : s.walls) w.fhydro = v3(0, 0, 0);
    const size_t A = s.activeNodes.size();
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)A; ++k) {
        const size_t i = s.activeNodes[k];
        std::memcpy(&s.fs[i * Q], &s.f[i * Q], sizeof(double) * Q);
    }
    int bad = 0;
    const bool mbb = s.P.coupling == HB_MOVING_BB;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (long k = 0; k < (long)A; ++k) {
        const size_t i = s.activeNodes[k];
        if (mbb && s.inside[i]) continue;  // solid
        double* fi = &s.f[i * Q];
        const double* fsi = &s.fs[i * Q];
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[i * Q + j];
            const uint8_t t = s.type[l];
            if ((t == 0 || t == 3) && mbb && s.inside[l]) {  // moving bounce-back on the particle
                const double BBi = 6.0 * s.n[i] * W[j] * dot(mbbVelocity(s, l), cvec(j));
                fi[OPP[j]] = fsi[j] - BBi;
            } else if (t == 0 || t == 3) {
                fi[OPP[j]] = s.fs[(size_t)l * Q + OPP[j]];
            } else if (t == 2) {  // constant-pressure gas link
                const double usq = norm2(s.u[i]);
                const double vuj = dot(s.u[i], cvec(j));
                fi[OPP[j]] = -fsi[j] + W[j] * 1.0 * (2.0 + 9.0 * (vuj * vuj) - 3.0 * usq);
            } else if (t == 8) {
                const double BBi = 6.0 * s.n[i] * W[j] * dot(s.u[l], cvec(j));
                fi[OPP[j]] = fsi[j] - BBi;
            } else if (t == 7) {
                fi[OPP[j]] = fsi[j];
            } else if (t == 9) {  // curved walls, LB.cpp:1278-1319 (curve: node.cpp:458-472)
                const V3 vel = s.u[l];
                const double BBi = 2.0 * 3.0 * 1.0 * 1.0 * s.n[i] * W[j] * dot(vel, cvec(j));
                const double dl = s.delta[(size_t)l * Q + OPP[j]];
                const double tau = 0.5 + 3.0 * s.visc[i];
                const double chi = dl >= 0.5 ? (2.0 * dl - 1.0) / tau : (2.0 * dl - 1.0) / (tau - 2.0);
                V3 ubf = v3(0.0, 0.0, 0.0);
                if (dl >= 0.5) {
                    ubf = add(mul((dl - 1) / dl, s.u[i]), mul(1 / dl, vel));
                } else {
                    const uint32_t back = s.nb[i * Q + OPP[j]];
                    ubf = (s.type[back] == 0 && s.has[back]) ? s.u[back] : vel;
                }
                const double usq = norm2(s.u[i]);
                const double vu = dot(s.u[i], cvec(j));
                const double fStar = s.n[i] * W[j] * (1 + 3.0 * dot(cvec(j), ubf) + 4.5 * vu * vu + 1.5 * usq);
                fi[OPP[j]] = (1.0 - chi) * fsi[j] + chi * fStar - BBi;
            } else if (t == 5 || t == 6) {  // slip walls, LB.cpp:1358-1456
                // moving slip walls (6) bounce back with BBi of the wall node's velocity
                const double BBi = t == 6 ? 6.0 * s.n[i] * W[j] * dot(s.u[l], cvec(j)) : 0.0;
                const double S1 = s.P.slip_coefficient, S2 = 1.0 - s.P.slip_coefficient;
                int c = -1, d = 0;
                if (j > 6) {  // diagonal links: specular reflection when one side is open
                    const SlipPair sp = slip_pair(j);
                    const uint32_t c1 = s.nb[i * Q + sp.check[0]], c2 = s.nb[i * Q + sp.check[1]];
                    const bool a1 = s.isActive(c1), a2 = s.isActive(c2);
                    if (a1 && !a2) { c = (int)c1; d = sp.dir[0]; }
                    else if (!a1 && a2) { c = (int)c2; d = sp.dir[1]; }
                }
                if (c >= 0)
                    fi[OPP[j]] = t == 6 ? S1 * s.fs[(size_t)c * Q + d] + S2 * (fsi[j] - BBi)
                                        : S1 * s.fs[(size_t)c * Q + d] + S2 * fsi[j];
                else
                    fi[OPP[j]] = t == 6 ? fsi[j] - BBi : fsi[j];
            } else {
                bad += 1;
            }
        }
    }
    if (bad) return fail("TYPE ERROR: link to an unsupported node type");
    if (mbb) mbbForces(s);
    // moving-wall force and extra mass in the reference's ordered node order (LB.cpp:1321-1341)
    double extraMass = 0.0;
    for (size_t k = 0; k < A; ++k) {
        const size_t i = s.activeNodes[k];
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[i * Q + j];
            if (s.type[l] != 8) continue;
            const double BBi = 6.0 * s.n[i] * W[j] * dot(s.u[l], cvec(j));
            const double sc = (2.0 * (s.fs[i * Q + j] - 1.0 * W[j]) - BBi) * 1.0;
            Wall& w = s.walls[s.solid[l]];
            w.fhydro = add(w.fhydro, mul(sc, cvec(j)));
            extraMass += BBi * s.mass[i];
        }
    }
    const double add_m = extraMass / (double)s.interfaceNodes.size();  // redistributeMass
    for (uint32_t i : s.interfaceNodes) s.mass[i] += add_m;
    return true;
}

bool lbStep(hbo_sim& s) {  // LB::latticeBolzmannStep, LB.cpp:221-233
    cleanLists(s);
    const size_t A = s.activeNodes.size();
    const bool mbb = s.P.coupling == HB_MOVING_BB;  // nodes inside particles are solid
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)A; ++k)
        if (!(mbb && s.inside[s.activeNodes[k]])) reconstruct(s, s.activeNodes[k]);
    if (mbb) {
        for (size_t k = 0; k < A; ++k) s.hf[s.activeNodes[k]] = v3(0, 0, 0);
    } else {
        computeHydroForces(s);
    }
    if (!s.P.force_field) s.lbF = v3(0, 0, 0);  // LB.cpp:1074-1076
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)A; ++k)
        if (!(mbb && s.inside[s.activeNodes[k]])) collideNode(s, s.activeNodes[k]);
    return streaming(s);
}

// ---- free surface (LB.cpp:1492-1804) -----------------------------------------------

void updateMass(hbo_sim& s) {  // LB.cpp:1492-1590
    for (uint32_t i : s.interfaceNodes) s.newMass[i] = s.mass[i];
    for (uint32_t i : s.interfaceNodes) {
        double dm = 0.0;
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[(size_t)i * Q + j];
            double a = 0.0;
            const uint8_t t = s.type[l];
            if (t == 3) a = 0.5 * (s.mass[l] + s.mass[i]);
            else if (t == 0) a = 1.0;
            else if (t == 2) a = 0.0;
            else if (t == 8 || t == 9) a = 1.0 * s.mass[i];
            else if (t == 6) {  // moving slip wall; a static slip wall (5) has no branch: 0
                bool mixed = false;
                if (j > 6) {
                    const SlipPair sp = slip_pair(j);
                    const bool a1 = s.isActive(s.nb[(size_t)i * Q + sp.check[0]]);
                    const bool a2 = s.isActive(s.nb[(size_t)i * Q + sp.check[1]]);
                    mixed = a1 != a2;
                }
                a += mixed ? 1.0 * (1.0 - s.P.slip_coefficient) * s.mass[i] : 1.0 * s.mass[i];
            }
            dm += 1.0 * a * (s.f[(size_t)i * Q + OPP[j]] - s.fs[(size_t)i * Q + j]);
        }
        s.newMass[i] += dm;
    }
    for (uint32_t i : s.fluidNodes) s.mass[i] = s.n[i];
    for (uint32_t i : s.interfaceNodes) s.mass[i] = s.newMass[i];
}

void eraseValue(std::vector<uint32_t>& v, uint32_t x) {
    for (long k = (long)v.size() - 1; k >= 0; --k)
        if (v[k] == x) v.erase(v.begin() + k);
}

void updateInterface(hbo_sim& s) {  // LB.cpp:1592-1804
    double surplus = 0.0;
    std::vector<uint32_t> filled, emptied, newIf;
    for (long k = (long)s.interfaceNodes.size() - 1; k >= 0; --k) {  // findInterfaceMutants
        const uint32_t i = s.interfaceNodes[k];
        if (s.mass[i] > s.n[i]) {
            filled.push_back(i);
            s.type[i] = 0;
            s.fluidNodes.push_back(i);
            s.interfaceNodes.erase(s.interfaceNodes.begin() + k);
        } else if (s.mass[i] < 0.0) {
            emptied.push_back(i);
            s.type[i] = 2;
            s.interfaceNodes.erase(s.interfaceNodes.begin() + k);
        }
    }
    for (uint32_t i : filled) {  // smoothenInterface, gas neighbours of filled cells
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[(size_t)i * Q + j];
            if (s.type[l] == 2) {
                s.type[l] = 3;
                newIf.push_back(l);
                nodeInit(s, l, 1.0, s.u[i], 0.01 * 1.0, s.visc[i], add(s.hf[i], s.lbF));
                s.hf[l] = v3(0, 0, 0);
                surplus -= 0.01 * 1.0;
            }
        }
    }
    for (uint32_t i : emptied) {  // fluid neighbours of emptied cells
        for (int j = 0; j < Q; ++j) {
            const uint32_t l = s.nb[(size_t)i * Q + j];
            if (s.type[l] == 0) {
                s.type[l] = 3;
                newIf.push_back(l);
                s.mass[l] = 0.99 * s.n[l];
                surplus += 0.01 * s.n[l];
                eraseValue(s.fluidNodes, l);
            }
        }
    }
    auto contains = [](const std::vector<uint32_t>& v, uint32_t x) {
        return std::find(v.begin(), v.end(), x) != v.end();
    };
    for (uint32_t i : emptied) {  // updateMutants
        if (!contains(newIf, i)) {
            surplus += s.mass[i];
            s.has[i] = 0;
        }
    }
    for (uint32_t i : filled) {
        if (!contains(newIf, i)) {
            surplus += s.mass[i] - s.n[i];
            s.mass[i] = s.n[i];
        }
    }
    for (uint32_t i : newIf) s.interfaceNodes.push_back(i);
    for (long k = (long)s.interfaceNodes.size() - 1; k >= 0; --k) {  // removeIsolated
        const uint32_t i = s.interfaceNodes[k];
        bool sf = true;
        for (int j = 1; j < Q; ++j)
            if (s.type[s.nb[(size_t)i * Q + j]] == 2) { sf = false; break; }
        if (sf) {
            surplus += s.mass[i] - s.n[i];
            s.mass[i] = s.n[i];
            s.type[i] = 0;
            s.interfaceNodes.erase(s.interfaceNodes.begin() + k);
            s.fluidNodes.push_back(i);
        }
    }
    for (long k = (long)s.interfaceNodes.size() - 1; k >= 0; --k) {
        const uint32_t i = s.interfaceNodes[k];
        bool sg = true;
        for (int j = 1; j < Q; ++j)
            if (s.type[s.nb[(size_t)i * Q + j]] == 0) { sg = false; break; }
        if (sg) {
            surplus += s.mass[i];
            s.interfaceNodes.erase(s.interfaceNodes.begin() + k);
            s.type[i] = 2;
            s.has[i] = 0;
        }
    }
    const double add_m = surplus / (double)s.interfaceNodes.size();  // redistributeMass
    for (uint32_t i : s.interfaceNodes) s.mass[i] += add_m;
}

// ---- coupling (LB.cpp:1921-2033) ----------------------------------------------------

// the first particle of the element (its spheres, then its ghosts) that covers pt, or -1
int coveringComponent(const hbo_sim& s, unsigned cluster, V3 pt) {
    for (unsigned c : s.comps[cluster]) {
        const Part& q = s.parts[c];
        if (norm2(sub(pt, q.x0)) < q.r * q.r) return (int)c;  // insideSphere, vector.cpp:153-158
    }
    return -1;
}

// LB::latticeBoltzmannCouplingStep (LB.cpp:247-280): updateIndices after a neighbour
// rebuild with periodic faces (LB.cpp:1826-1849: initializeParticleBoundaries over every
// particle, then resetLists), findNewActive, findNewSolid
void couplingStep(hbo_sim& s) {
    if (s.newNeighborList) {
        for (size_t i = 0; i < s.N; ++i) {
            s.inside[i] = 0;
            if (!s.isActive(i)) continue;
            for (size_t n = 0; n < s.parts.size(); ++n)
                if (norm2(sub(s.pos(i), s.parts[n].x0)) < s.parts[n].r * s.parts[n].r) {
                    s.inside[i] = 1;
                    s.solid[i] = (uint32_t)n;
                }
        }
        s.particleNodes.clear();
        for (size_t i = 0; i < s.N; ++i)
            if (s.inside[i]) s.particleNodes.push_back((uint32_t)i);
        s.newNeighborList = false;
    }
    std::vector<uint32_t> pop;
    for (uint32_t i : s.particleNodes) {  // findNewActive
        if (coveringComponent(s, s.parts[s.solid[i]].cluster, s.pos(i)) < 0) {
            pop.push_back(i);
            s.inside[i] = 0;
        }
    }
    for (uint32_t i : pop) eraseValue(s.particleNodes, i);
    for (size_t k = 0; k < s.particleNodes.size(); ++k) {  // findNewSolid (list grows)
        const uint32_t i = s.particleNodes[k];
        const unsigned cl = s.parts[s.solid[i]].cluster;
        for (int kk = 1; kk < 7; ++kk) {
            const uint32_t l = s.nb[(size_t)i * Q + kk];
            if (s.inside[l]) continue;
            const int c = coveringComponent(s, cl, s.pos(l));
            if (c >= 0) {
                s.solid[l] = (uint32_t)c;
                s.inside[l] = 1;
                s.particleNodes.push_back(l);
            }
        }
    }
    if (s.P.coupling != HB_MOVING_BB) return;
    // Moving bounce-back: a node the particle uncovered (and no particle covers again)
    // becomes fluid with f = f_eq(rho, u), u the velocity the particle had at the node, rho
    // the mean density of its fluid links that were fluid before this step, in link order
    // (1 without any).  Nodes a particle covered keep their populations unused.
    std::vector<uint8_t> popped(s.N, 0);
    for (uint32_t i : pop) popped[i] = 1;
    std::vector<double> rho(pop.size(), 1.0);
    std::vector<V3> vel(pop.size());
    for (size_t k = 0; k < pop.size(); ++k) {
        const uint32_t i = pop[k];
        if (s.inside[i]) continue;
        double sum = 0.0;
        int cnt = 0;
        for (int j = 1; j < Q; ++j) {
            const uint32_t l = s.nb[(size_t)i * Q + j];
            if (l == i || !s.isActive(l) || s.inside[l] || popped[l]) continue;
            sum += s.n[l];
            ++cnt;
        }
        if (cnt) rho[k] = sum / (double)cnt;
        vel[k] = mbbVelocity(s, i);  // solid[i] still names the particle that left
    }
    for (size_t k = 0; k < pop.size(); ++k) {
        const uint32_t i = pop[k];
        if (s.inside[i]) continue;
        const V3 uu = vel[k];
        const double usq = norm2(uu);
        for (int j = 0; j < Q; ++j) {
            const double vu = dot(uu, cvec(j));
            s.f[(size_t)i * Q + j] = W[j] * rho[k] * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
        }
        s.n[i] = rho[k];
    }
}

}  // namespace

extern "C" {

const char* hbo_last_error(void) { return g_err.c_str(); }

int hbo_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#endif
    return 0;
}

hbo_sim* hbo_create(const hb_params* p, const hb_elements* e, const hb_objects* o) {
    return hbo_create_cyl(p, e, o, nullptr);
}

hbo_sim* hbo_create_cyl(const hb_params* p, const hb_elements* e, const hb_objects* o, const hb_cylinders* cy) {
    if (!p) { g_err = "null params"; return nullptr; }
    hbo_sim* s = new hbo_sim();
    if (cy) {
        for (int k = 0; k < cy->count; ++k) {
            Cyl c;
            c.p1 = v3(cy->p1[3 * k], cy->p1[3 * k + 1], cy->p1[3 * k + 2]);
            c.p2 = v3(cy->p2[3 * k], cy->p2[3 * k + 1], cy->p2[3 * k + 2]);
            const V3 ax = sub(c.p2, c.p1);
            const double nrm = std::sqrt(norm2(ax));
            c.naxes = v3(ax.x / nrm, ax.y / nrm, ax.z / nrm);
            c.R = cy->radius[k];
            c.omega = cy->omega ? v3(cy->omega[3 * k], cy->omega[3 * k + 1], cy->omega[3 * k + 2]) : v3(0, 0, 0);
            c.moving = cy->moving ? cy->moving[k] != 0 : false;
            s->cyl.push_back(c);
        }
    }
    s->P = *p;
    s->X = p->lb_size[0]; s->Y = p->lb_size[1]; s->Z = p->lb_size[2];
    s->N = (size_t)s->X * s->Y * s->Z;
    s->lbF = v3(p->lbF[0], p->lbF[1], p->lbF[2]);
    s->demF = s->lbF;  // DEM.cpp:194, captured before collision may zero lbF
    if (o) {
        for (int k = 0; k < o->count; ++k) {
            Object ob;
            ob.r = o->radius[k];
            ob.x0 = v3(o->x0[k], o->x0[o->count + k], o->x0[2 * o->count + k]);
            ob.x1 = o->x1 ? v3(o->x1[k], o->x1[o->count + k], o->x1[2 * o->count + k]) : v3(0, 0, 0);
            ob.fparticle = v3(0, 0, 0);
            s->obj.push_back(ob);
        }
    }
    buildWalls(*s);
    // elements (DEM.cpp:185-297, elmt.cpp:13-61)
    const double re = p->restitution;
    s->dampCoeff = -1.0 * std::sqrt(2.0) * std::log(re) / std::sqrt((std::log(re) * std::log(re) + M_PI));
    s->knConst = 2.0 / 3.0 * p->young_mod / (1 - p->poisson * p->poisson);
    s->ksConst = 2.0 * p->young_mod / (2.0 - p->poisson) / (1.0 + p->poisson);
    const int ne = e ? e->count : 0;
    for (int k = 0; k < ne; ++k) {
        Elmt el;
        std::memset(&el, 0, sizeof(el));
        el.radius = e->radius[k];
        el.x0 = v3(e->x0[k], e->x0[ne + k], e->x0[2 * ne + k]);
        el.x1 = e->x1 ? v3(e->x1[k], e->x1[ne + k], e->x1[2 * ne + k]) : v3(0, 0, 0);
        el.w0 = e->w0 ? v3(e->w0[k], e->w0[ne + k], e->w0[2 * ne + k]) : v3(0, 0, 0);
        el.q0 = e->q0 ? Quat{e->q0[k], e->q0[ne + k], e->q0[2 * ne + k], e->q0[3 * ne + k]} : Quat{1, 0, 0, 0};
        el.xp0 = el.x0;
        el.xp1 = el.x1;
        el.qp0 = el.q0;
        el.wpGlobal = el.wGlobal = el.wpLocal = el.wLocal = el.w0;
        el.size = e->size ? e->size[k] : 1;
        if (el.size < 1 || el.size > 4) { g_err = "element size outside 1..4"; delete s; return nullptr; }
        const double sm = 4.0 / 3.0 * p->density * M_PI * el.radius * el.radius * el.radius;
        el.m = el.size * sm;  // elmt.cpp:62-71, Huygens-Steiner over the prototype positions
        el.I = mul(el.size * 2.0 / 5.0 * sm * el.radius * el.radius, v3(1.0, 1.0, 1.0));
        for (int n = 0; n < el.size; ++n) {
            const V3 t = prototype(el.size, n);
            el.I = add(el.I, mul(sm * el.radius * el.radius, v3(t.y * t.y + t.z * t.z, t.z * t.z + t.x * t.x,
                                                               t.x * t.x + t.y * t.y)));
        }
        s->el.push_back(el);
    }
    // particles (elmt::generateParticles, elmt.cpp:122-137), in element order
    s->comps.assign(ne, {});
    for (int k = 0; k < ne; ++k)
        for (int n = 0; n < s->el[k].size; ++n) {
            Part q;
            q.cluster = (unsigned)k;
            q.proto = n;
            q.r = s->el[k].radius;
            q.x0 = q.x1 = q.radiusVec = v3(0, 0, 0);
            s->comps[k].push_back((unsigned)s->parts.size());
            s->parts.push_back(q);
        }
    s->stdParticles = (unsigned)s->parts.size();
    updateParticles(*s, false);
    // periodic face pairs (DEM::initializePbcs, DEM.cpp:937-989)
    const int L[3] = {s->X, s->Y, s->Z};
    for (int k = 0; k < 3; ++k) {
        if (p->boundary[2 * k] != 4) continue;
        if (p->boundary[2 * k + 1] != 4) { g_err = "periodic boundary on one face only"; delete s; return nullptr; }
        Pbc b;
        b.p = v3(k == 0 ? 0.5 : 0.0, k == 1 ? 0.5 : 0.0, k == 2 ? 0.5 : 0.0);
        b.v = v3(k == 0 ? L[0] - 2.0 : 0.0, k == 1 ? L[1] - 2.0 : 0.0, k == 2 ? L[2] - 2.0 : 0.0);
        b.p1 = b.p;
        b.p2 = add(b.p, b.v);
        b.n1 = divs(b.v, norm(b.v));
        b.n2 = mul(-1.0, b.n1);
        s->pbcs.push_back(b);
    }
    s->stdObjects = (unsigned)s->obj.size();
    s->deltat = ne ? 1.0 / double(p->multi_step) : 1.0;
    s->demTime = 0.0;
    s->maxDisp = 0.0;
    s->nebrRange = 0.0;
    s->triggerSet = false;
    if (ne) {
        initNeighborParameters(*s);
        // periodicObjects (DEM.cpp:990-1063): images of the objects near the faces
        std::vector<Ghost> og;
        for (const Pbc& b : s->pbcs)
            for (unsigned k = 0; k < s->stdObjects; ++k) {
                const double ld = b.dist1(s->obj[k].x0), rd = b.dist2(s->obj[k].x0);
                if (ld < 2.0 * s->nebrRange && ld > 0.0) og.push_back(Ghost{k, b.v});
                else if (rd < 2.0 * s->nebrRange && rd > 0.0) og.push_back(Ghost{k, mul(-1.0, b.v)});
            }
        const size_t ns = og.size();
        for (size_t g1 = 0; g1 < ns; ++g1)
            for (size_t g2 = g1 + 1; g2 < ns; ++g2)
                if (og[g1].index == og[g2].index) og.push_back(Ghost{og[g1].index, add(og[g1].vec, og[g2].vec)});
        for (const Ghost& g : og) {
            Object ob = s->obj[g.index];
            ob.x0 = add(ob.x0, g.vec);
            s->obj.push_back(ob);
        }
        evalNeighborTable(*s);
    }
    if (!buildLattice(*s, e, o)) { delete s; return nullptr; }
    return s;
}

void hbo_destroy(hbo_sim* s) { delete s; }

int hbo_dem_step(hbo_sim* s) {
    const int ms = s->el.empty() ? 1 : s->P.multi_step;
    for (int k = 0; k < ms; ++k) {
        if (s->el.empty()) { s->demTime += s->deltat; continue; }
        demSubstep(*s);
    }
    return 0;
}
int hbo_fs_step(hbo_sim* s) {
    updateMass(*s);
    updateInterface(*s);
    return 0;
}
int hbo_coupling_step(hbo_sim* s) {
    couplingStep(*s);
    return 0;
}
int hbo_lb_step(hbo_sim* s) { return lbStep(*s) ? 0 : 1; }

int hbo_cycle(hbo_sim* s, int nsteps) {  // goCycle, hybird.cpp:35-66
    for (int t = 0; t < nsteps; ++t) {
        if (s->P.dem_solve) hbo_dem_step(s);
        if (!s->P.lb_solve) continue;
        if (s->P.free_surface) hbo_fs_step(s);
        if (s->P.dem_solve) hbo_coupling_step(s);
        if (hbo_lb_step(s)) return 1;
    }
    return 0;
}

int64_t hbo_nodes(const hbo_sim* s) { return (int64_t)s->N; }
int64_t hbo_active(const hbo_sim* s) {
    int64_t a = 0;
    for (size_t i = 0; i < s->N; ++i) a += s->isActive(i) ? 1 : 0;
    return a;
}

int hbo_get_lattice(const hbo_sim* s, uint8_t* type, uint8_t* inside, uint32_t* solid,
                    uint8_t* has_node, double* f, double* n, double* u, double* mass, double* visc,
                    double* hydro_force) {
    const size_t N = s->N;
    for (size_t i = 0; i < N; ++i) {
        if (type) type[i] = s->type[i];
        if (inside) inside[i] = s->inside[i];
        if (solid) solid[i] = s->solid[i];
        if (has_node) has_node[i] = s->has[i];
        if (f)
            for (int j = 0; j < Q; ++j) f[j * N + i] = s->f[i * Q + j];
        if (n) n[i] = s->n[i];
        if (u) { u[i] = s->u[i].x; u[N + i] = s->u[i].y; u[2 * N + i] = s->u[i].z; }
        if (mass) mass[i] = s->mass[i];
        if (visc) visc[i] = s->visc[i];
        if (hydro_force) { hydro_force[i] = s->hf[i].x; hydro_force[N + i] = s->hf[i].y; hydro_force[2 * N + i] = s->hf[i].z; }
    }
    return 0;
}

int hbo_set_lattice(hbo_sim* s, const double* f, const double* n, const double* u,
                    const double* mass, const double* visc) {
    const size_t N = s->N;
    for (size_t i = 0; i < N; ++i) {
        if (f)
            for (int j = 0; j < Q; ++j) s->f[i * Q + j] = f[j * N + i];
        if (n) s->n[i] = n[i];
        if (u) s->u[i] = v3(u[i], u[N + i], u[2 * N + i]);
        if (mass) s->mass[i] = mass[i];
        if (visc) s->visc[i] = visc[i];
    }
    return 0;
}

// problem code changing lb.lbF between steps: the collision reads it every step
// (LB.cpp:1098-1111); zero without forceFieldSolve (LB.cpp:1074-1076); demF keeps the
// value captured at init (DEM.cpp:194)
int hbo_set_body_force(hbo_sim* s, const double* force) {
    s->lbF = s->P.force_field ? v3(force[0], force[1], force[2]) : v3(0, 0, 0);
    return 0;
}

int hbo_get_elements(const hbo_sim* s, double* x0, double* x1, double* w, double* q0,
                     double* fhydro, double* mhydro, double* fparticle, double* fwall,
                     double* mparticle, double* mwall, double* fluid_volume) {
    const size_t E = s->el.size();
    auto put = [E](double* dst, size_t k, V3 v) {
        if (!dst) return;
        dst[k] = v.x; dst[E + k] = v.y; dst[2 * E + k] = v.z;
    };
    for (size_t k = 0; k < E; ++k) {
        const Elmt& e = s->el[k];
        put(x0, k, e.x0); put(x1, k, e.x1); put(w, k, e.wGlobal);
        if (q0) { q0[k] = e.q0.q0; q0[E + k] = e.q0.q1; q0[2 * E + k] = e.q0.q2; q0[3 * E + k] = e.q0.q3; }
        put(fhydro, k, e.FHydro); put(mhydro, k, e.MHydro); put(fparticle, k, e.FParticle);
        put(fwall, k, e.FWall); put(mparticle, k, e.MParticle); put(mwall, k, e.MWall);
        if (fluid_volume) fluid_volume[k] = e.fluidVolume;
    }
    return 0;
}

int64_t hbo_get_pairs(const hbo_sim* s, uint32_t* pairs, int64_t capacity) {
    const int64_t np = (int64_t)s->neighborTable.size() / 2;
    if (pairs)
        for (int64_t k = 0; k < std::min(np, capacity) * 2; ++k) pairs[k] = s->neighborTable[k];
    return np;
}

int64_t hbo_get_interface(const hbo_sim* s, uint32_t* cells, int64_t capacity) {
    const int64_t c = (int64_t)s->interfaceNodes.size();
    if (cells)
        for (int64_t k = 0; k < std::min(c, capacity); ++k) cells[k] = s->interfaceNodes[k];
    return c;
}

int hbo_get_walls(const hbo_sim* s, double* fhydro, double* fparticle, int32_t* nwalls) {
    const size_t W0 = s->walls.size();
    if (nwalls) *nwalls = (int32_t)W0;
    for (size_t k = 0; k < W0; ++k) {
        if (fhydro) { fhydro[3 * k] = s->walls[k].fhydro.x; fhydro[3 * k + 1] = s->walls[k].fhydro.y; fhydro[3 * k + 2] = s->walls[k].fhydro.z; }
        if (fparticle) { fparticle[3 * k] = s->walls[k].fparticle.x; fparticle[3 * k + 1] = s->walls[k].fparticle.y; fparticle[3 * k + 2] = s->walls[k].fparticle.z; }
    }
    return 0;
}

int hbo_get_objects(const hbo_sim* s, double* fparticle, int32_t* nobjects) {
    const size_t O = s->obj.size();
    if (nobjects) *nobjects = (int32_t)O;
    for (size_t k = 0; k < O && fparticle; ++k) {
        fparticle[3 * k] = s->obj[k].fparticle.x;
        fparticle[3 * k + 1] = s->obj[k].fparticle.y;
        fparticle[3 * k + 2] = s->obj[k].fparticle.z;
    }
    return 0;
}

double hbo_total_mass(const hbo_sim* s) {
    double m = 0.0;
    for (size_t i = 0; i < s->N; ++i)
        if (s->isActive(i) && !s->inside[i]) m += s->mass[i];
    return m;
}

int hbo_dem_scalars(const hbo_sim* s, double* out) {
    out[0] = s->demTime; out[1] = s->maxDisp; out[2] = s->nebrRange; out[3] = s->deltat;
    return 0;
}

// Drag on the objects along one axis from the post-collision populations of the last
// step: node::bounceBackForce (node.cpp:283-291) with BBi = 0, (2 (fs_j - w_j rho0)) c_j,
// summed over every link from an active node to a static wall node inside an object
// sphere (the node set LB.cpp:535-550 turns into walls), in node order.
double hbo_object_drag(const hbo_sim* s, int axis) {
    std::vector<uint8_t> isObj(s->N, 0);
    for (size_t i = 0; i < s->N; ++i) {
        if (s->type[i] != 7) continue;
        for (const Object& ob : s->obj)
            if (norm2(sub(s->pos(i), ob.x0)) < ob.r * ob.r) { isObj[i] = 1; break; }
    }
    double J = 0.0;
    for (size_t i = 0; i < s->N; ++i) {
        if (!s->isActive(i)) continue;
        for (int j = 1; j < Q; ++j) {
            if (!isObj[s->nb[i * Q + j]]) continue;
            const V3 c = cvec(j);
            const double ca = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            J += 2.0 * (s->fs[i * Q + j] - W[j] * 1.0) * ca;
        }
    }
    return J;
}

}  // extern "C"
