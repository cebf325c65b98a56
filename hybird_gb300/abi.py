"""ctypes mirror of include/hybird_gpu.h.

The library's boundary is the C-ABI in include/hybird_gpu.h; this module only gives
Python callers (tests, bench.py) the same structs and a loader.  No computation
happens here.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libhybird_gpu.so")

HB_OK = 0
HB_ERR_ARG, HB_ERR_UNSUPPORTED, HB_ERR_CUDA, HB_ERR_NOMEM = 1, 2, 3, 4
HB_ERR_CAPACITY, HB_ERR_STATE, HB_ERR_NUMERIC = 5, 6, 7
HB_FP64, HB_FP32, HB_FP16S = 0, 1, 2
HB_BGK, HB_TRT = 0, 1
HB_LINEAR, HB_HERTZIAN = 0, 1
HB_DIRECT_FORCING, HB_MOVING_BB = 0, 1

STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_UNSUPPORTED", 3: "ERR_CUDA", 4: "ERR_NOMEM",
                5: "ERR_CAPACITY", 6: "ERR_STATE", 7: "ERR_NUMERIC"}


class HbParams(C.Structure):
    _fields_ = [
        ("lb_size", C.c_int32 * 3),
        ("boundary", C.c_int32 * 6),
        ("units", C.c_double * 3),
        ("init_visc", C.c_double),
        ("init_velocity", C.c_double * 3),
        ("lbF", C.c_double * 3),
        ("force_field", C.c_int32),
        ("non_newtonian", C.c_int32),
        ("plastic_visc", C.c_double),
        ("yield_stress", C.c_double),
        ("turbulence", C.c_int32),
        ("turb_const", C.c_double),
        ("free_surface", C.c_int32),
        ("collision", C.c_int32),
        ("trt_magic", C.c_double),
        ("precision", C.c_int32),
        ("gas_box", C.c_double * 2),
        ("lb_solve", C.c_int32),
        ("dem_solve", C.c_int32),
        ("multi_step", C.c_int32),
        ("contact_model", C.c_int32),
        ("density", C.c_double),
        ("linear_stiff", C.c_double),
        ("young_mod", C.c_double),
        ("poisson", C.c_double),
        ("restitution", C.c_double),
        ("visc_tang", C.c_double),
        ("friction_part", C.c_double),
        ("friction_wall", C.c_double),
        ("num_visc", C.c_double),
        ("cap_neighbors", C.c_int64),
        ("cap_interface", C.c_int64),
        ("slip_coefficient", C.c_double),
        ("coupling", C.c_int32),
    ]


class HbElements(C.Structure):
    _fields_ = [("count", C.c_int32), ("radius", C.POINTER(C.c_double)),
                ("x0", C.POINTER(C.c_double)), ("x1", C.POINTER(C.c_double)),
                ("w0", C.POINTER(C.c_double)), ("q0", C.POINTER(C.c_double)),
                ("size", C.POINTER(C.c_int32))]


class HbObjects(C.Structure):
    _fields_ = [("count", C.c_int32), ("radius", C.POINTER(C.c_double)),
                ("x0", C.POINTER(C.c_double)), ("x1", C.POINTER(C.c_double))]


class HbStatus(C.Structure):
    _fields_ = [("numeric_error", C.c_int32), ("capacity_error", C.c_int32),
                ("unsupported_link", C.c_int32), ("reserved", C.c_int32),
                ("interface_cells", C.c_int64), ("active_nodes", C.c_int64),
                ("pairs", C.c_int64), ("contacts", C.c_int64),
                ("mass_surplus", C.c_double), ("total_mass", C.c_double)]


class HbExport(C.Structure):
    _fields_ = [("max_fluid_speed", C.c_double), ("total_fluid_mass", C.c_double),
                ("plastic_percent", C.c_double), ("active_nodes", C.c_int64),
                ("plastic_nodes", C.c_int64), ("max_particle_speed", C.c_double),
                ("max_particle_spin", C.c_double), ("collision_force", C.c_double),
                ("hydraulic_force", C.c_double), ("particle_mass", C.c_double),
                ("object_force", C.c_double * 3), ("energy_kin", C.c_double),
                ("energy_rot_kin", C.c_double), ("energy_tr_kin", C.c_double),
                ("energy_grav", C.c_double), ("energy_total", C.c_double)]


class HbAdjointCfg(C.Structure):
    _fields_ = [("steps", C.c_int32), ("checkpoint_every", C.c_int32), ("precision", C.c_int32),
                ("drag_axis", C.c_int32), ("tau", C.c_double), ("body_force", C.c_double * 3),
                ("inlet_velocity", C.POINTER(C.c_double))]


def dptr(a):
    """double* of a C-contiguous float64 array (or NULL for None)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_params(lb_size, boundary, init_visc=0.1, lbF=(0.0, 0.0, 0.0), force_field=1,
                init_velocity=(0.0, 0.0, 0.0), non_newtonian=0, plastic_visc=0.0,
                yield_stress=0.0, turbulence=0, turb_const=0.0, free_surface=0,
                collision=HB_BGK, trt_magic=3.0 / 16.0, precision=HB_FP64, gas_box=(0.0, 0.0),
                lb_solve=1, dem_solve=1, multi_step=1, contact_model=HB_LINEAR, density=2.5,
                linear_stiff=1e3, young_mod=1.0, poisson=0.3, restitution=0.8, visc_tang=0.5,
                friction_part=0.5, friction_wall=0.5, num_visc=0.0, cap_neighbors=0, cap_interface=0,
                slip_coefficient=0.0, coupling=0):
    p = HbParams()
    p.lb_size[:] = list(lb_size)
    p.boundary[:] = list(boundary)
    p.units[:] = [1.0, 1.0, 1.0]
    p.init_visc = init_visc
    p.init_velocity[:] = list(init_velocity)
    p.lbF[:] = list(lbF)
    p.force_field = force_field
    p.non_newtonian = non_newtonian
    p.plastic_visc = plastic_visc
    p.yield_stress = yield_stress
    p.turbulence = turbulence
    p.turb_const = turb_const
    p.free_surface = free_surface
    p.collision = collision
    p.trt_magic = trt_magic
    p.precision = precision
    p.gas_box[:] = list(gas_box)
    p.lb_solve = lb_solve
    p.dem_solve = dem_solve
    p.multi_step = multi_step
    p.contact_model = contact_model
    p.density = density
    p.linear_stiff = linear_stiff
    p.young_mod = young_mod
    p.poisson = poisson
    p.restitution = restitution
    p.visc_tang = visc_tang
    p.friction_part = friction_part
    p.friction_wall = friction_wall
    p.num_visc = num_visc
    p.cap_neighbors = cap_neighbors
    p.cap_interface = cap_interface
    p.slip_coefficient = slip_coefficient
    p.coupling = coupling
    return p


class HbCylinders(C.Structure):
    _fields_ = [("count", C.c_int32), ("p1", C.POINTER(C.c_double)), ("p2", C.POINTER(C.c_double)),
                ("radius", C.POINTER(C.c_double)), ("omega", C.POINTER(C.c_double)),
                ("moving", C.POINTER(C.c_int32))]


class CylinderArrays:
    """Keeps the buffers behind an HbCylinders struct alive.  Rows: p1 (3), p2 (3), R,
    optionally omega (3) and moving."""

    def __init__(self, rows):
        r = [list(map(float, row)) for row in rows]
        n = len(r)
        self.p1 = np.array([x[0:3] for x in r]).reshape(-1)
        self.p2 = np.array([x[3:6] for x in r]).reshape(-1)
        self.R = np.array([x[6] for x in r])
        self.om = np.array([x[7:10] if len(x) >= 10 else [0.0, 0.0, 0.0] for x in r]).reshape(-1)
        self.mv = np.array([int(x[10]) if len(x) >= 11 else 0 for x in r], dtype=np.int32)
        self.cy = HbCylinders(n, dptr(self.p1), dptr(self.p2), dptr(self.R), dptr(self.om),
                              self.mv.ctypes.data_as(C.POINTER(C.c_int32)))

    def ptr(self):
        return C.byref(self.cy)


class ElementArrays:
    """Keeps the numpy buffers alive behind an HbElements / HbObjects struct."""

    def __init__(self, spheres=None, objects=None, sizes=None, quats=None):
        """spheres: [n, 4] (x, y, z, radius) per element; sizes: spheres per element
        (1..4, multi-sphere prototypes), quats: [n, 4] orientations (default identity)."""
        self.el = None
        self.ob = None
        if spheres is not None and len(spheres):
            s = np.asarray(spheres, dtype=np.float64).reshape(-1, 4)
            n = len(s)
            self.radius = np.ascontiguousarray(s[:, 3])
            self.x0 = np.ascontiguousarray(s[:, :3].T.reshape(-1))
            self.x1 = np.zeros(3 * n)
            self.w0 = np.zeros(3 * n)
            self.q0 = None if quats is None else np.ascontiguousarray(np.asarray(quats, np.float64).reshape(-1, 4).T.reshape(-1))
            self.size = None if sizes is None else np.ascontiguousarray(np.asarray(sizes, np.int32).reshape(-1))
            self.el = HbElements(n, dptr(self.radius), dptr(self.x0), dptr(self.x1), dptr(self.w0),
                                 None if self.q0 is None else dptr(self.q0),
                                 None if self.size is None else self.size.ctypes.data_as(C.POINTER(C.c_int32)))
        if objects is not None and len(objects):
            o = np.asarray(objects, dtype=np.float64).reshape(-1, 4)
            m = len(o)
            self.oradius = np.ascontiguousarray(o[:, 3])
            self.ox0 = np.ascontiguousarray(o[:, :3].T.reshape(-1))
            self.ox1 = np.zeros(3 * m)
            self.ob = HbObjects(m, dptr(self.oradius), dptr(self.ox0), dptr(self.ox1))

    def el_ptr(self):
        return C.byref(self.el) if self.el is not None else None

    def ob_ptr(self):
        return C.byref(self.ob) if self.ob is not None else None
