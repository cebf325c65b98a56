"""Test infrastructure: ctypes access to the CPU oracle (oracle/hb_oracle.cpp) and to
the reference fixtures in tests/golden/.  Only tests, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module."""
import ctypes as C
import json
import os
import subprocess

import numpy as np

from hybird_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
ORACLE_SO = os.path.join(REPO, "oracle", "_build", "libhb_oracle.so")

_lib = None


def oracle_lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(ORACLE_SO):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "port"], check=True,
                       stdout=subprocess.DEVNULL)
    lib = C.CDLL(ORACLE_SO)
    P = C.POINTER
    lib.hbo_create.restype = C.c_void_p
    lib.hbo_create.argtypes = [P(abi.HbParams), P(abi.HbElements), P(abi.HbObjects)]
    lib.hbo_create_cyl.argtypes = [P(abi.HbParams), P(abi.HbElements), P(abi.HbObjects), P(abi.HbCylinders)]
    lib.hbo_create_cyl.restype = C.c_void_p
    lib.hbo_destroy.argtypes = [C.c_void_p]
    lib.hbo_last_error.restype = C.c_char_p
    for name in ("hbo_cycle",):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int]
    for name in ("hbo_dem_step", "hbo_fs_step", "hbo_coupling_step", "hbo_lb_step"):
        getattr(lib, name).argtypes = [C.c_void_p]
    lib.hbo_nodes.restype = C.c_int64
    lib.hbo_nodes.argtypes = [C.c_void_p]
    lib.hbo_active.restype = C.c_int64
    lib.hbo_active.argtypes = [C.c_void_p]
    lib.hbo_get_lattice.argtypes = [C.c_void_p] + [C.c_void_p] * 10
    lib.hbo_set_lattice.argtypes = [C.c_void_p] + [C.c_void_p] * 5
    lib.hbo_set_body_force.argtypes = [C.c_void_p, C.c_void_p]
    lib.hbo_get_elements.argtypes = [C.c_void_p] + [C.c_void_p] * 11
    lib.hbo_get_pairs.restype = C.c_int64
    lib.hbo_get_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    lib.hbo_get_interface.restype = C.c_int64
    lib.hbo_get_interface.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    lib.hbo_get_walls.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbo_get_objects.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbo_total_mass.restype = C.c_double
    lib.hbo_total_mass.argtypes = [C.c_void_p]
    lib.hbo_dem_scalars.argtypes = [C.c_void_p, C.c_void_p]
    lib.hbo_set_threads.argtypes = [C.c_int]
    lib.hbo_object_drag.restype = C.c_double
    lib.hbo_object_drag.argtypes = [C.c_void_p, C.c_int]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleSim:
    """One CPU-oracle simulation (FP64, reference semantics)."""

    def __init__(self, params, spheres=None, objects=None, threads=1, cylinders=None, sizes=None, quats=None):
        self.lib = oracle_lib()
        self.lib.hbo_set_threads(threads)
        self.params = params
        self.arrays = abi.ElementArrays(spheres, objects, sizes, quats)
        self.cyl = abi.CylinderArrays(cylinders) if cylinders is not None and len(cylinders) else None
        self.h = self.lib.hbo_create_cyl(C.byref(params), self.arrays.el_ptr(), self.arrays.ob_ptr(),
                                         self.cyl.ptr() if self.cyl else None)
        if not self.h:
            raise RuntimeError("oracle init failed: " + self.lib.hbo_last_error().decode())
        self.N = int(self.lib.hbo_nodes(self.h))
        self.E = 0 if self.arrays.el is None else self.arrays.el.count

    def close(self):
        if self.h:
            self.lib.hbo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def cycle(self, n=1):
        rc = self.lib.hbo_cycle(self.h, n)
        if rc:
            raise RuntimeError("oracle step failed: " + self.lib.hbo_last_error().decode())

    def lattice(self):
        N = self.N
        out = dict(type=np.zeros(N, np.uint8), inside=np.zeros(N, np.uint8),
                   solid=np.zeros(N, np.uint32), has_node=np.zeros(N, np.uint8),
                   f=np.zeros(19 * N), n=np.zeros(N), u=np.zeros(3 * N), mass=np.zeros(N),
                   visc=np.zeros(N), hydroForce=np.zeros(3 * N))
        self.lib.hbo_get_lattice(self.h, *[_p(out[k]) for k in
                                           ("type", "inside", "solid", "has_node", "f", "n", "u",
                                            "mass", "visc", "hydroForce")])
        return out

    def set_lattice(self, f=None, n=None, u=None, mass=None, visc=None):
        self.lib.hbo_set_lattice(self.h, _p(f), _p(n), _p(u), _p(mass), _p(visc))

    def set_body_force(self, force):
        f = np.ascontiguousarray(force, dtype=np.float64)
        self.lib.hbo_set_body_force(self.h, f.ctypes.data_as(C.c_void_p))

    def object_drag(self, axis=0):
        return self.lib.hbo_object_drag(self.h, axis)

    def set_inlet(self, inlet):
        """Moving-wall nodes of the planes x = 0 and x = X-1 move along x with
        inlet[y + Y*z] (the node velocity the moving-wall bounce-back reads)."""
        X, Y, Z = self.params.lb_size
        lat = self.lattice()
        u = lat["u"].reshape(3, Z, Y, X).copy()
        t = lat["type"].reshape(Z, Y, X)
        uin = np.asarray(inlet, dtype=np.float64).reshape(Z, Y)
        for xp in (0, X - 1):
            m = t[:, :, xp] == 8
            u[0, :, :, xp][m] = uin[m]
            u[1, :, :, xp][m] = 0.0
            u[2, :, :, xp][m] = 0.0
        self.set_lattice(u=np.ascontiguousarray(u.reshape(-1)))

    def elements(self):
        E = self.E
        keys = ("x0", "x1", "w", "q0", "FHydro", "MHydro", "FParticle", "FWall", "MParticle",
                "MWall", "fluidVolume")
        out = {k: np.zeros((4 if k == "q0" else 1 if k == "fluidVolume" else 3) * E) for k in keys}
        self.lib.hbo_get_elements(self.h, *[_p(out[k]) for k in keys])
        return out

    def pairs(self):
        n = self.lib.hbo_get_pairs(self.h, None, 0)
        buf = np.zeros(2 * max(n, 1), np.uint32)
        self.lib.hbo_get_pairs(self.h, _p(buf), n)
        return buf[:2 * n]

    def interface(self):
        n = self.lib.hbo_get_interface(self.h, None, 0)
        buf = np.zeros(max(n, 1), np.uint32)
        self.lib.hbo_get_interface(self.h, _p(buf), n)
        return buf[:n]

    def walls(self):
        nw = C.c_int32(0)
        self.lib.hbo_get_walls(self.h, None, None, C.byref(nw))
        fh = np.zeros(3 * max(nw.value, 1))
        fp = np.zeros(3 * max(nw.value, 1))
        self.lib.hbo_get_walls(self.h, _p(fh), _p(fp), C.byref(nw))
        return fh[:3 * nw.value], fp[:3 * nw.value]

    def objects(self):
        no = C.c_int32(0)
        self.lib.hbo_get_objects(self.h, None, C.byref(no))
        fp = np.zeros(3 * max(no.value, 1))
        self.lib.hbo_get_objects(self.h, _p(fp), C.byref(no))
        return fp[:3 * no.value]

    def total_mass(self):
        return self.lib.hbo_total_mass(self.h)


# ------------------------------------------------------------------------------------
# reference fixtures
# ------------------------------------------------------------------------------------

def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def golden_params(d, **over):
    """hb_params equivalent to the .cfg the reference ran for this fixture."""
    c = json.loads(bytes(d["params_json"]).decode())
    kw = dict(
        lb_size=(c["lbSizeX"], c["lbSizeY"], c["lbSizeZ"]),
        boundary=tuple(c[f"boundary{k}"] for k in range(6)),
        init_visc=c["initVisc"],
        lbF=(c["lbFX"], c["lbFY"], c["lbFZ"]),
        force_field=c["forceFieldSolve"],
        init_velocity=(c["initVelocityX"], c["initVelocityY"], c["initVelocityZ"]),
        non_newtonian=c["nonNewtonianSolve"], plastic_visc=c["plasticVisc"],
        yield_stress=c["yieldStress"], turbulence=c["turbulenceSolve"], turb_const=c["turbConst"],
        free_surface=c["freeSurfaceSolve"], lb_solve=c["lbSolve"], dem_solve=c["demSolve"], multi_step=c["multiStep"],
        contact_model=abi.HB_LINEAR if c["contactModel"] == "LINEAR" else abi.HB_HERTZIAN,
        density=c["density"], linear_stiff=c["linearStiff"], young_mod=c["youngMod"],
        poisson=c["poisson"], restitution=c["restitution"], visc_tang=c["viscTang"],
        friction_part=c["frictionCoefPart"], friction_wall=c["frictionCoefWall"],
        num_visc=c["numVisc"], slip_coefficient=c["slipCoefficient"],
    )
    if "gasbox" in c:
        kw["gas_box"] = tuple(c["gasbox"])
    kw.update(over)
    return abi.make_params(**kw)


def golden_cylinders(d):
    """The cylinder rows a fixture was made with (p1, p2, R), or None."""
    c = json.loads(bytes(d["params_json"]).decode())
    return [c["cylinder"]] if "cylinder" in c else None


def golden_gasbox(name):
    return {"dambreak_fs": (0.4, 0.6), "dambreak_slip": (0.4, 0.6)}.get(name, (0.0, 0.0))


def rel_linf(a, b, mask=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if mask is not None:
        a, b = a[..., mask], b[..., mask]
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)
