"""Generate the parity fixtures in this folder from the reference hybird code itself.

Test infrastructure only.  For every case below this script writes a .cfg file (the
reference's own GetPot format) plus particle/object files, runs ``oracle/_ref/ref_dump``
(the unmodified reference sources, built by ``make -C oracle ref``) with
OMP_NUM_THREADS=1 -- coupled force sums in the reference are thread-order dependent
(LB.cpp:1897) -- and stores the reference's FP64 state at the listed step counts as a
compressed ``<case>.npz``, with the reference's output-step quantities (``io_values``:
maximum fluid speed, IO::totFluidMass, IO::totPlastic, active count, maximum particle
speed and spin, IO::collisionForceTot, IO::hydraulicForceTot, IO::totParticleMass,
IO::totForceObject, particle energies kin/rotKin/trKin/grav/total) and, for the steps
listed under ``vtk``, the text of IO::exportParaviewFluidOld and of
IO::exportRecycleParticles.

Run in a container that has the reference tree:

    make -C oracle ref && python tests/golden/make_golden.py

The fixtures are committed; the GPU host never runs this script.
"""
import json
import os
import random
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")

# ----------------------------------------------------------------------------------
# cases
# ----------------------------------------------------------------------------------

BASE = dict(
    problemName="NONE", demSolve=1, lbSolve=1, freeSurfaceSolve=0, forceFieldSolve=1,
    nonNewtonianSolve=0, turbulenceSolve=0, unitLength=1.0, unitTime=1.0, unitDensity=1.0,
    initVisc=0.1, plasticVisc=0.0, yieldStress=0.0, turbConst=0.0, slipCoefficient=0.0,
    initVelocityX=0.0, initVelocityY=0.0, initVelocityZ=0.0,
    lbFX=0.0, lbFY=0.0, lbFZ=0.0, maxTime=1e9, maximumTimeSteps=0, screenExpTime=0.0,
    fluidExpTime=0.0, partExpTime=0.0, objectExpTime=0.0, recycleExpTime=0.0, saveCount=0,
    demInitialRepeat=0.0, lbmInitialRepeat=0, density=2.5, contactModel="LINEAR",
    youngMod=1.0, poisson=0.3, linearStiff=1e3, restitution=0.8, viscTang=0.5,
    frictionCoefPart=0.5, frictionCoefWall=0.5, numVisc=0.0, multiStep=1, criticalRatio=0.1,
    scale=1.0, translateX=0.0, translateY=0.0, translateZ=0.0,
)


def rsa_spheres(seed, n, rmin, rmax, lo, hi, gap=0.0):
    """Seeded random sequential addition of non-overlapping spheres inside [lo+r, hi-r]^3."""
    rng = random.Random(seed)
    out = []
    tries = 0
    while len(out) < n and tries < 200000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = [rng.uniform(lo[k] + r, hi[k] - r) for k in range(3)]
        ok = True
        for (q, rq) in out:
            d2 = sum((c[k] - q[k]) ** 2 for k in range(3))
            if d2 < (r + rq + gap) ** 2:
                ok = False
                break
        if ok:
            out.append((c, r))
    return out


def rsa_periodic(seed, n, rmin, rmax, lo, hi, period, gap=0.3):
    """Seeded random sequential addition with centres uniform in [lo, hi] (not shrunk by
    r) and overlaps checked through the minimum image along the axes with a period."""
    rng = random.Random(seed)
    out = []
    tries = 0
    while len(out) < n and tries < 200000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = [rng.uniform(lo[k], hi[k]) for k in range(3)]
        ok = True
        for (q, rq) in out:
            d2 = 0.0
            for k in range(3):
                d = c[k] - q[k]
                if period[k]:
                    d -= period[k] * round(d / period[k])
                d2 += d * d
            if d2 < (r + rq + gap) ** 2:
                ok = False
                break
        if ok:
            out.append((c, r))
    return out


CASES = {
    # periodic-x/z channel with walls at y=0/Ly-1 (the 64x32x32 channel workload, shrunk)
    "channel_bgk": dict(
        cfg=dict(lbSizeX=12, lbSizeY=8, lbSizeZ=6, lbFX=2e-5, initVisc=0.1,
                 boundary0=4, boundary1=4, boundary2=7, boundary3=7, boundary4=4, boundary5=4),
        spheres=[], objects=[], steps=[0, 1, 5, 40], full=[0, 1, 40]),
    # moving-wall bounce-back at y+ (type 8; the reference's walls have zero speed) and
    # static wall at y-, non-zero initial velocity so the wall force is exercised
    "channel_movwall": dict(
        cfg=dict(lbSizeX=10, lbSizeY=8, lbSizeZ=6, lbFX=1e-5, lbFZ=-3e-6, initVisc=0.05,
                 initVelocityX=0.01, initVelocityZ=0.004,
                 boundary0=4, boundary1=4, boundary2=7, boundary3=8, boundary4=4, boundary5=4),
        spheres=[], objects=[], steps=[0, 1, 12], full=[0, 1, 12]),
    # Bingham + Smagorinsky inline viscosity (node.cpp:103-145)
    "channel_bingham_smag": dict(
        cfg=dict(lbSizeX=10, lbSizeY=8, lbSizeZ=6, lbFX=4e-5, initVisc=0.1,
                 nonNewtonianSolve=1, plasticVisc=1.0 / 30.0, yieldStress=3e-6,
                 turbulenceSolve=1, turbConst=0.01,
                 boundary0=4, boundary1=4, boundary2=7, boundary3=7, boundary4=4, boundary5=4),
        spheres=[], objects=[], steps=[0, 1, 10], full=[0, 1, 10], vtk=[10]),
    # closed box with a few spheres: DEM + direct-forcing coupling (LB.cpp:1851-2033)
    "box_spheres": dict(
        cfg=dict(lbSizeX=16, lbSizeY=14, lbSizeZ=16, lbFZ=-2e-4, initVisc=0.1, multiStep=3,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("rsa", 11, 7, 2.2, 3.2), objects=[], steps=[0, 1, 2, 10, 30], full=[1, 30], vtk=[30]),
    # DEM only (no LB): spheres against walls and fixed objects (DEM.cpp:1668-2136)
    "dem_objects": dict(
        # particles stay > nebrRange from the side walls: the reference keeps only the
        # first wall in range per particle (DEM.cpp:1502-1511) and would let corner
        # particles fall through the floor
        cfg=dict(lbSizeX=32, lbSizeY=32, lbSizeZ=32, lbSolve=0, lbFZ=-1e-3, multiStep=20,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("rsa", 5, 14, 1.6, 2.6, (9.5, 9.5, 6.0), (22.5, 22.5, 28.0)),
        objects=[(13.0, 14.0, 4.0, 3.0), (19.0, 17.0, 3.5, 2.5)],
        steps=[0, 1, 50, 100, 150], full=[], vtk=[50]),
    # slip walls (LB.cpp:1358-1456): static slip at y-, moving slip at y+, periodic x/z
    "channel_slip": dict(
        cfg=dict(lbSizeX=12, lbSizeY=8, lbSizeZ=6, lbFX=2e-5, lbFZ=-4e-6, initVisc=0.08,
                 slipCoefficient=0.35, initVelocityX=0.01, initVelocityY=0.002,
                 boundary0=4, boundary1=4, boundary2=5, boundary3=6, boundary4=4, boundary5=4),
        spheres=[], objects=[], steps=[0, 1, 5, 30], full=[1, 30]),
    # closed box of slip walls with particles (contacts with slip walls, DEM.cpp:442-471)
    "box_slip": dict(
        cfg=dict(lbSizeX=14, lbSizeY=12, lbSizeZ=14, lbFX=3e-5, lbFZ=-2e-4, initVisc=0.1,
                 slipCoefficient=0.6, multiStep=3,
                 boundary0=5, boundary1=7, boundary2=5, boundary3=5, boundary4=6, boundary5=5),
        spheres=("rsa", 13, 4, 2.0, 2.6), objects=[], steps=[0, 1, 10, 40], full=[1, 40]),
    # free surface against static slip walls (updateMass has no slip-static branch)
    "dambreak_slip": dict(
        cfg=dict(lbSizeX=20, lbSizeY=8, lbSizeZ=12, lbFZ=-5e-4, initVisc=0.05, freeSurfaceSolve=1,
                 slipCoefficient=0.5,
                 boundary0=5, boundary1=7, boundary2=7, boundary3=5, boundary4=5, boundary5=7),
        spheres=[], objects=[], gasbox=(0.4, 0.6), steps=[0, 1, 5, 20, 60], full=[1, 20, 60]),
    # curved walls (LB.cpp:552-603, 1278-1319): a pipe along x, periodic ends
    "pipe_curved": dict(
        cfg=dict(lbSizeX=10, lbSizeY=12, lbSizeZ=12, lbFX=2e-5, initVisc=0.1, initVelocityX=0.005,
                 boundary0=4, boundary1=4, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=[], objects=[], cylinder=(0.0, 5.5, 5.3, 1.0, 5.5, 5.3, 4.6),
        steps=[0, 1, 5, 30], full=[1, 30], vtk=[30]),
    # coupled: spheres settling in a fluid-filled horizontal pipe closed at both ends
    # (curved walls + cylinder contacts + coupling)
    "pipe_spheres": dict(
        cfg=dict(lbSizeX=14, lbSizeY=16, lbSizeZ=16, lbFZ=-2e-4, initVisc=0.1, multiStep=3,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("rsa", 23, 5, 1.6, 2.2, (1.5, 4.5, 3.5), (12.5, 10.5, 10.5)), objects=[],
        cylinder=(0.0, 7.5, 7.5, 1.0, 7.5, 7.5, 6.8), steps=[0, 1, 10, 40], full=[1, 40]),
    # DEM only: spheres falling inside a horizontal cylinder (DEM.cpp:1535-1550, 1719-2058)
    "dem_cylinder": dict(
        cfg=dict(lbSizeX=24, lbSizeY=20, lbSizeZ=20, lbSolve=0, lbFZ=-2e-3, multiStep=20,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("rsa", 21, 8, 1.2, 1.8, (4.0, 7.0, 5.0), (20.0, 13.0, 9.0)),
        objects=[], cylinder=(0.0, 10.0, 10.0, 1.0, 10.0, 10.0, 8.6), steps=[0, 1, 30, 60, 100], full=[]),
    # Hertzian contacts (DEM.cpp:2138-2222): spheres falling onto the floor and onto each
    # other, DEM only; kept > nebrRange from the side walls (first wall in range only)
    "dem_hertz": dict(
        cfg=dict(lbSizeX=28, lbSizeY=28, lbSizeZ=40, lbSolve=0, lbFZ=-2e-3, multiStep=20,
                 contactModel="HERTZIAN", youngMod=5e3, poisson=0.3,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("rsa", 9, 10, 1.5, 2.2, (8.5, 8.5, 1.6), (19.5, 19.5, 30.0)),
        objects=[], steps=[0, 1, 30, 60, 100], full=[], vtk=[60]),
    # periodic DEM (DEM.cpp:937-1063, 1395-1411, 1554-1664): spheres under a tilted gravity
    # cross the periodic x and y faces; DEM only
    "dem_periodic": dict(
        cfg=dict(lbSizeX=24, lbSizeY=20, lbSizeZ=28, lbSolve=0, lbFX=1e-3, lbFY=-6e-4, lbFZ=-2e-3,
                 multiStep=20,
                 boundary0=4, boundary1=4, boundary2=4, boundary3=4, boundary4=7, boundary5=7),
        spheres=("rsa_periodic", 31, 14, 1.4, 2.0, (0.6, 0.6, 3.0), (22.4, 18.4, 22.0), (22.0, 18.0, 0.0)),
        objects=[], steps=[0, 1, 30, 60, 100, 150], full=[]),
    # fixed objects near the periodic faces get images across them (DEM.cpp:990-1063);
    # spheres driven along x meet them through the faces, DEM only
    "dem_periodic_objects": dict(
        cfg=dict(lbSizeX=24, lbSizeY=20, lbSizeZ=20, lbSolve=0, lbFX=3e-3, lbFZ=-5e-4, multiStep=20,
                 boundary0=4, boundary1=4, boundary2=4, boundary3=4, boundary4=7, boundary5=7),
        spheres=("rsa_periodic", 33, 6, 1.4, 1.8, (15.0, 7.5, 3.5), (20.5, 12.5, 8.0), (22.0, 18.0, 0.0)),
        objects=[(1.5, 10.0, 5.5, 2.2), (12.0, 10.0, 2.5, 1.5)],
        steps=[0, 1, 30, 60, 90, 120], full=[]),
    # the same with the lattice: ghost particles cover the nodes across the periodic faces
    # and every neighbour rebuild re-marks the particle nodes (LB.cpp:1826-1849)
    "box_periodic": dict(
        cfg=dict(lbSizeX=18, lbSizeY=16, lbSizeZ=18, lbFX=1.5e-3, lbFY=-1e-3, lbFZ=-1e-3, initVisc=0.1,
                 multiStep=3,
                 boundary0=4, boundary1=4, boundary2=4, boundary3=4, boundary4=7, boundary5=7),
        spheres=("rsa_periodic", 37, 9, 1.6, 2.2, (0.6, 0.6, 4.0), (16.4, 14.4, 13.0), (16.0, 14.0, 0.0)),
        objects=[], steps=[0, 1, 2, 10, 40, 80, 120], full=[1, 120], vtk=[80]),
    # multi-sphere elements (DEM.cpp:404-433, elmt.cpp:17-137): clusters of 1-4 spheres
    # falling onto the floor, a fixed object and each other, DEM only; kept > nebrRange
    # from the side walls (first wall in range only, DEM.cpp:1502-1511)
    "dem_clusters": dict(
        cfg=dict(lbSizeX=40, lbSizeY=40, lbSizeZ=40, lbSolve=0, lbFX=3e-4, lbFZ=-2e-3, multiStep=20,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("clusters", 41, 12, 1.2, 1.7, (6.5, 6.5, 1.0), (33.0, 33.0, 38.0)),
        objects=[(20.0, 20.0, 5.0, 3.0)], steps=[0, 1, 30, 60, 100, 150], full=[]),
    # the same shapes in a fluid with periodic x (ghost copies of cluster spheres)
    "box_clusters": dict(
        cfg=dict(lbSizeX=20, lbSizeY=18, lbSizeZ=20, lbFX=8e-4, lbFZ=-8e-4, initVisc=0.1, multiStep=3,
                 boundary0=4, boundary1=4, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=("clusters", 43, 8, 1.6, 2.0, (0.6, 1.0, 1.0), (19.4, 17.0, 17.0)),
        objects=[], steps=[0, 1, 2, 10, 40, 80], full=[1, 80], vtk=[40]),
    # free-surface dam break (LB.cpp:1492-1804), column x < 0.4 Lx, z < 0.6 Lz
    "dambreak_fs": dict(
        cfg=dict(lbSizeX=20, lbSizeY=8, lbSizeZ=12, lbFZ=-5e-4, initVisc=0.05, freeSurfaceSolve=1,
                 boundary0=7, boundary1=7, boundary2=7, boundary3=7, boundary4=7, boundary5=7),
        spheres=[], objects=[], gasbox=(0.4, 0.6), steps=[0, 1, 2, 5, 20, 60, 150], full=[0, 1, 20, 150],
        vtk=[60]),
}


def write_cfg(path, cfg):
    with open(path, "w") as fh:
        for k, v in cfg.items():
            fh.write(f"{k} = {v}\n")


def write_particles(path, spheres, sizes=None, quats=None):
    with open(path, "w") as fh:
        fh.write(f"{len(spheres)}\n")
        for i, (c, r) in enumerate(spheres):
            size = 1 if sizes is None else int(sizes[i])
            q = (1.0, 0.0, 0.0, 0.0) if quats is None else tuple(quats[i])
            vals = [i, size, repr(r), repr(c[0]), repr(c[1]), repr(c[2]), 0.0, 0.0, 0.0,
                    0.0, 0.0, 0.0, repr(q[0]), repr(q[1]), repr(q[2]), repr(q[3]), 0.0, 0.0, 0.0, 0.0]
            fh.write(" ".join(str(v) for v in vals) + "\n")


def cluster_elements(seed, n, rmin, rmax, lo, hi):
    """Seeded multi-sphere elements (1 to 4 spheres, DEM.cpp:404-433 prototypes) with
    random unit orientations, placed so that their bounding spheres (radius 2r) do not
    overlap."""
    rng = random.Random(seed)
    out = []
    tries = 0
    while len(out) < n and tries < 200000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        size = 1 + len(out) % 4
        c = [rng.uniform(lo[k] + 2 * r, hi[k] - 2 * r) for k in range(3)]
        if any(sum((c[k] - q[k]) ** 2 for k in range(3)) < (2 * r + 2 * rq + 0.3) ** 2 for (q, rq, _, _) in out):
            continue
        q = [rng.gauss(0.0, 1.0) for _ in range(4)]
        nq = sum(v * v for v in q) ** 0.5
        q = [v / nq for v in q]
        if q[0] < 0:
            q = [-v for v in q]
        out.append((c, r, size, q))
    return out


def write_objects(path, objects):
    with open(path, "w") as fh:
        fh.write(f"{len(objects)}\n")
        for i, (x, y, z, r) in enumerate(objects):
            vals = [i, 1, r, x, y, z, 0.0, 0.0, 0.0] + [0.0] * 11
            fh.write(" ".join(str(v) for v in vals) + "\n")


def parse_dump(path):
    """Return a list of dicts, one per dumped step."""
    dt = {0: np.float64, 1: np.uint32, 2: np.uint8, 3: np.int64}
    snaps = []
    with open(path, "rb") as fh:
        data = fh.read()
    off = 0
    cur = None
    while off < len(data):
        name = data[off:off + 32].split(b"\0")[0].decode()
        code, cnt = struct.unpack_from("<IQ", data, off + 32)
        off += 44
        arr = np.frombuffer(data, dtype=dt[code], count=cnt, offset=off).copy()
        off += cnt * np.dtype(dt[code]).itemsize
        if name == "header":
            cur = {}
            snaps.append(cur)
        cur[name] = arr
    return snaps


def run_case(name, spec):
    cfg = dict(BASE)
    cfg.update(spec["cfg"])
    sizes = (cfg["lbSizeX"], cfg["lbSizeY"], cfg["lbSizeZ"])
    sizes = quats = None
    if spec["spheres"] and spec["spheres"][0] == "clusters":
        els = cluster_elements(*spec["spheres"][1:])
        spheres = [(c, r) for (c, r, _, _) in els]
        sizes = [sz for (_, _, sz, _) in els]
        quats = [q for (_, _, _, q) in els]
    elif spec["spheres"] and spec["spheres"][0] == "rsa_periodic":
        spheres = rsa_periodic(*spec["spheres"][1:])
    elif spec["spheres"]:
        seed, n, rmin, rmax = spec["spheres"][1:5]
        lo, hi = (1.5, 1.5, 1.5), (sizes[0] - 2.5, sizes[1] - 2.5, sizes[2] - 2.5)
        if len(spec["spheres"]) > 5:
            lo, hi = spec["spheres"][5], spec["spheres"][6]
        spheres = rsa_spheres(seed, n, rmin, rmax, lo, hi, gap=0.3)
    else:
        spheres = []
    with tempfile.TemporaryDirectory() as tmp:
        cfg["particleFile"] = os.path.join(tmp, "particles.dat")
        cfg["objectFile"] = os.path.join(tmp, "objects.dat")
        write_particles(cfg["particleFile"], spheres, sizes, quats)
        write_objects(cfg["objectFile"], spec["objects"])
        cpath = os.path.join(tmp, "case.cfg")
        write_cfg(cpath, cfg)
        out = os.path.join(tmp, "out.bin")
        cmd = [REF_DUMP, cpath, os.path.join(tmp, "work"), out] + [str(s) for s in spec["steps"]]
        if spec.get("gasbox"):
            cmd += ["--gasbox", str(spec["gasbox"][0]), str(spec["gasbox"][1])]
        if spec.get("vtk"):
            cmd += ["--vtk"]
        if spec.get("cylinder"):
            cmd += ["--cylinder"] + [repr(v) for v in spec["cylinder"]]
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.run(cmd, check=True, cwd=tmp, env=env, stdout=subprocess.DEVNULL, timeout=120)
        snaps = parse_dump(out)

    store = {}
    params = {k: v for k, v in cfg.items() if k not in ("particleFile", "objectFile")}
    if spec.get("cylinder"):
        params["cylinder"] = list(spec["cylinder"])
    store["params_json"] = np.frombuffer(json.dumps(params).encode(), dtype=np.uint8)
    store["spheres"] = np.array([[c[0], c[1], c[2], r] for (c, r) in spheres], dtype=np.float64).reshape(-1, 4)
    store["objects"] = np.array(spec["objects"], dtype=np.float64).reshape(-1, 4)
    if sizes is not None:
        store["sizes"] = np.array(sizes, dtype=np.int32)
        store["quats"] = np.array(quats, dtype=np.float64).reshape(-1, 4)
    store["steps"] = np.array(spec["steps"], dtype=np.int64)
    lattice = cfg.get("lbSolve", 1) == 1
    for s in snaps:
        step = int(s["header"][0])
        p = f"s{step}_"
        store[p + "header"] = s["header"]
        if lattice:
            store[p + "type"] = s["type"]
            store[p + "inside"] = s["inside"]
            store[p + "solid"] = s["solid"]
            store[p + "has_node"] = s["has_node"]
            store[p + "n"] = s["n"]
            store[p + "u"] = s["u"]
            store[p + "mass"] = s["mass"]
            store[p + "visc"] = s["visc"]
            store[p + "interfaceNodes"] = s["interfaceNodes"]
            store[p + "particleNodes"] = s["particleNodes"]
            store[p + "totalMass"] = s["totalMass"]
            store[p + "w_FHydro"] = s["w_FHydro"]
            if step in spec["full"]:
                store[p + "f"] = s["f"]
                store[p + "hydroForce"] = s["hydroForce"]
            if step in spec.get("vtk", []):
                store[p + "vtk"] = s["vtk"]
        if step in spec.get("vtk", []) and "recycle" in s:
            store[p + "recycle"] = s["recycle"]
        for k in ("e_x0", "e_x1", "e_x2", "e_w", "e_q0", "e_FHydro", "e_MHydro", "e_FParticle",
                  "e_FWall", "e_MParticle", "e_MWall", "e_fluidVolume", "e_m", "e_I",
                  "neighborTable", "nearWallTable", "nearObjectTable", "w_FParticle",
                  "dem_scalars", "o_FParticle", "io_values", "ghost_index", "ghost_vec"):
            store[p + k] = s[k]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **store)
    return len(snaps)


def main(argv):
    if not os.path.exists(REF_DUMP):
        sys.exit("build the reference first: make -C oracle ref")
    names = argv[1:] or list(CASES)
    for name in names:
        n = run_case(name, CASES[name])
        print(f"{name}: {n} snapshots")


if __name__ == "__main__":
    main(sys.argv)
