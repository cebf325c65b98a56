"""Python handle on the CUDA library through its C-ABI (include/hybird_gpu.h).

Every call goes through ``_lib/libhybird_gpu.so``; there is no CPU fallback: loading
fails loudly when the library is missing.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_lib = None


class HbError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("HB_LIB_PATH", abi.LIB_PATH)  # an alternate build of the same ABI
    if not os.path.exists(path):
        raise HbError(f"CUDA library not built: {path} (run __graft_entry__.build())")
    L = C.CDLL(path)
    vp, P = C.c_void_p, C.POINTER
    L.hb_last_error.restype = C.c_char_p
    L.hb_create.argtypes = [P(abi.HbParams), P(vp)]
    L.hb_destroy.argtypes = [vp]
    L.hb_init.argtypes = [vp, P(abi.HbElements), P(abi.HbObjects)]
    L.hb_upload_lattice.argtypes = [vp] + [vp] * 8
    for name in ("hb_dem_step", "hb_fs_step", "hb_coupling_step", "hb_lb_step", "hb_synchronize"):
        getattr(L, name).argtypes = [vp]
    L.hb_cycle.argtypes = [vp, C.c_int32]
    L.hb_set_body_force.argtypes = [vp, vp]
    L.hb_download_lattice.argtypes = [vp] + [vp] * 9
    L.hb_download_elements.argtypes = [vp] + [vp] * 11
    L.hb_download_elements_async.argtypes = [vp] + [vp] * 11
    L.hb_host_register.argtypes = [vp, C.c_size_t]
    L.hb_host_unregister.argtypes = [vp]
    L.hb_set_element_sink.argtypes = [vp] + [vp] * 11
    L.hb_set_lattice_mirror.argtypes = [vp, C.c_int32]
    L.hb_download_pairs.argtypes = [vp, vp, C.c_int64, P(C.c_int64)]
    L.hb_download_ghosts.argtypes = [vp, vp, vp, C.c_int64, P(C.c_int64)]
    L.hb_download_interface.argtypes = [vp, vp, C.c_int64, P(C.c_int64)]
    L.hb_download_walls.argtypes = [vp, vp, vp, P(C.c_int32)]
    L.hb_download_objects.argtypes = [vp, vp, P(C.c_int32)]
    L.hb_export_values.argtypes = [vp, P(abi.HbExport)]
    L.hb_vtk_fluid_fields.argtypes = [vp] + [vp] * 6
    L.hb_write_vtk_fluid.argtypes = [vp, C.c_char_p]
    L.hb_get_params.argtypes = [vp, P(abi.HbParams), P(C.c_int32), P(C.c_int32)]
    L.hb_set_cylinders.argtypes = [vp, P(abi.HbCylinders)]
    L.hb_checkpoint_save.argtypes = [vp, C.c_char_p]
    L.hb_checkpoint_load.argtypes = [C.c_char_p, P(vp)]
    L.hb_write_recycle_particles.argtypes = [vp, C.c_char_p]
    L.hb_get_status.argtypes = [vp, P(abi.HbStatus)]
    L.hb_time_cycles.argtypes = [vp, C.c_int32, P(C.c_float), P(C.c_float), P(C.c_int32)]
    L.hb_profile_phases.argtypes = [vp, C.c_int32, vp, P(C.c_int32)]
    L.hb_adjoint_forward.argtypes = [vp, P(abi.HbAdjointCfg), vp]
    L.hb_adjoint_drag.argtypes = [vp, P(abi.HbAdjointCfg), vp, vp, vp, vp]
    L.hb_adjoint_timing.argtypes = [vp, P(C.c_float), P(C.c_float), P(C.c_int64), P(C.c_int64)]
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(rc):
    if rc != abi.HB_OK:
        raise HbError(f"{abi.STATUS_NAMES.get(rc, rc)}: {lib().hb_last_error().decode()}")


class GpuSim:
    """One simulation context on the current CUDA device."""

    def __init__(self, params, spheres=None, objects=None, cylinders=None, sizes=None, quats=None):
        self.L = lib()
        self.params = params
        self.arrays = abi.ElementArrays(spheres, objects, sizes, quats)
        h = C.c_void_p()
        check(self.L.hb_create(C.byref(params), C.byref(h)))
        self.h = h
        if cylinders is not None and len(cylinders):
            self.cyl = abi.CylinderArrays(cylinders)
            check(self.L.hb_set_cylinders(self.h, self.cyl.ptr()))
        check(self.L.hb_init(self.h, self.arrays.el_ptr(), self.arrays.ob_ptr()))
        X, Y, Z = params.lb_size
        self.N = X * Y * Z
        self.E = 0 if self.arrays.el is None else self.arrays.el.count

    def _adopt(self, L, h):
        """Wrap a context created by the library itself (hb_checkpoint_load)."""
        self.L, self.h = L, h
        self.params = abi.HbParams()
        ne, no = C.c_int32(0), C.c_int32(0)
        check(L.hb_get_params(h, C.byref(self.params), C.byref(ne), C.byref(no)))
        self.arrays = None
        X, Y, Z = self.params.lb_size
        self.N = X * Y * Z
        self.E = ne.value

    def close(self):
        if getattr(self, "h", None):
            self.L.hb_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def cycle(self, n=1):
        check(self.L.hb_cycle(self.h, n))
        check(self.L.hb_synchronize(self.h))

    def lattice(self, fields=None):
        """Node fields after the last step; `fields` limits the download (e.g. ("type", "n", "u"))."""
        N = self.N
        sizes = dict(type=(N, np.uint8), inside=(N, np.uint8), solid=(N, np.uint32), f=(19 * N, np.float64),
                     n=(N, np.float64), u=(3 * N, np.float64), mass=(N, np.float64), visc=(N, np.float64),
                     hydroForce=(3 * N, np.float64))
        keys = ("type", "inside", "solid", "f", "n", "u", "mass", "visc", "hydroForce")
        want = keys if fields is None else tuple(fields)
        out = {k: np.zeros(sizes[k][0], sizes[k][1]) for k in want}
        check(self.L.hb_download_lattice(self.h, *[_p(out.get(k)) for k in keys]))
        return out

    def upload(self, type, inside, solid, f, n, u, mass, visc=None):
        check(self.L.hb_upload_lattice(self.h, _p(type), _p(inside), _p(solid), _p(f), _p(n),
                                       _p(u), _p(mass), _p(visc)))

    def elements(self):
        E = self.E
        keys = ("x0", "x1", "w", "q0", "FHydro", "MHydro", "FParticle", "FWall", "MParticle",
                "MWall", "fluidVolume")
        out = {k: np.zeros((4 if k == "q0" else 1 if k == "fluidVolume" else 3) * E) for k in keys}
        check(self.L.hb_download_elements(self.h, *[_p(out[k]) for k in keys]))
        return out

    def pairs(self):
        n = C.c_int64(0)
        check(self.L.hb_download_pairs(self.h, None, 0, C.byref(n)))
        buf = np.zeros(2 * max(n.value, 1), np.uint32)
        check(self.L.hb_download_pairs(self.h, _p(buf), n.value, C.byref(n)))
        return buf[:2 * n.value]

    def ghosts(self):
        """Ghost particles of the last rebuild: (particle each copies [G], shift [G, 3])."""
        n = C.c_int64(0)
        check(self.L.hb_download_ghosts(self.h, None, None, 0, C.byref(n)))
        o = np.zeros(max(n.value, 1), np.uint32)
        v = np.zeros(3 * max(n.value, 1))
        check(self.L.hb_download_ghosts(self.h, _p(o), _p(v), n.value, C.byref(n)))
        return o[:n.value], v[:3 * n.value].reshape(-1, 3)

    def interface(self):
        n = C.c_int64(0)
        check(self.L.hb_download_interface(self.h, None, 0, C.byref(n)))
        buf = np.zeros(max(n.value, 1), np.uint32)
        check(self.L.hb_download_interface(self.h, _p(buf), n.value, C.byref(n)))
        return buf[:n.value]

    def walls(self):
        nw = C.c_int32(0)
        fh = np.zeros(18)
        fp = np.zeros(18)
        check(self.L.hb_download_walls(self.h, _p(fh), _p(fp), C.byref(nw)))
        return fh[:3 * nw.value], fp[:3 * nw.value]

    def objects(self):
        """objects[].FParticle of the last substep, [3*O] (x, y, z per object)."""
        no = C.c_int32(0)
        check(self.L.hb_download_objects(self.h, None, C.byref(no)))
        fp = np.zeros(3 * max(no.value, 1))
        check(self.L.hb_download_objects(self.h, _p(fp), C.byref(no)))
        return fp[:3 * no.value]

    def export_values(self):
        """The export.dat quantities of the current state (hb_export) as a dict."""
        e = abi.HbExport()
        check(self.L.hb_export_values(self.h, C.byref(e)))
        out = {k: getattr(e, k) for k, _ in abi.HbExport._fields_}
        out["object_force"] = np.array(e.object_force[:])
        return out

    def vtk_fields(self):
        """Per-node arrays of the fluid image-data file (type, v [N,3], pressure, dynVisc,
        mass, solidIndex)."""
        N = self.N
        out = {"type": np.zeros(N, np.int8), "v": np.zeros(3 * N), "pressure": np.zeros(N),
               "dyn_visc": np.zeros(N), "mass": np.zeros(N), "solid_index": np.zeros(N, np.uint32)}
        check(self.L.hb_vtk_fluid_fields(self.h, *[_p(out[k]) for k in
                                                   ("type", "v", "pressure", "dyn_visc", "mass", "solid_index")]))
        out["v"] = out["v"].reshape(N, 3)
        return out

    def write_vtk(self, path):
        check(self.L.hb_write_vtk_fluid(self.h, str(path).encode()))

    def save(self, path):
        """Full-state checkpoint (hb_checkpoint_save)."""
        check(self.L.hb_checkpoint_save(self.h, str(path).encode()))

    def write_recycle(self, path):
        check(self.L.hb_write_recycle_particles(self.h, str(path).encode()))

    @classmethod
    def load(cls, path):
        """A simulation restored from a checkpoint file (hb_checkpoint_load)."""
        L = lib()
        h = C.c_void_p()
        check(L.hb_checkpoint_load(str(path).encode(), C.byref(h)))
        g = cls.__new__(cls)
        g._adopt(L, h)
        return g

    def status(self):
        s = abi.HbStatus()
        check(self.L.hb_get_status(self.h, C.byref(s)))
        return s

    def profile_phases(self, n):
        us = np.zeros(64)
        k = C.c_int32(0)
        check(self.L.hb_profile_phases(self.h, n, _p(us), C.byref(k)))
        return us[:k.value]

    def time_cycles(self, n):
        tot, lbk, kpc = C.c_float(0), C.c_float(0), C.c_int32(0)
        check(self.L.hb_time_cycles(self.h, n, C.byref(tot), C.byref(lbk), C.byref(kpc)))
        return tot.value, lbk.value, kpc.value

    # ---- adjoint (reverse) entry points -------------------------------------------------
    def _adjoint_cfg(self, steps, checkpoint_every, precision, tau, force, inlet, axis):
        Y, Z = self.params.lb_size[1], self.params.lb_size[2]
        self._inlet = None if inlet is None else np.ascontiguousarray(inlet, dtype=np.float64).reshape(-1)
        if self._inlet is not None and self._inlet.size != Y * Z:
            raise ValueError(f"inlet field must hold Y*Z = {Y * Z} values")
        cfg = abi.HbAdjointCfg()
        cfg.steps, cfg.checkpoint_every, cfg.precision, cfg.drag_axis = steps, checkpoint_every, precision, axis
        cfg.tau = tau
        cfg.body_force[:] = list(force)
        cfg.inlet_velocity = abi.dptr(self._inlet)
        return cfg

    def adjoint_forward(self, steps, tau, force, inlet=None, precision=abi.HB_FP64, checkpoint_every=100, axis=0):
        """Object drag J after `steps` steps from the current state."""
        cfg = self._adjoint_cfg(steps, checkpoint_every, precision, tau, force, inlet, axis)
        J = np.zeros(1)
        check(self.L.hb_adjoint_forward(self.h, C.byref(cfg), _p(J)))
        return float(J[0])

    def adjoint_drag(self, steps, tau, force, inlet=None, precision=abi.HB_FP64, checkpoint_every=100, axis=0):
        """J and (dJ/dF[3], dJ/dtau, dJ/du_in[Y*Z]) by the reverse kernel."""
        cfg = self._adjoint_cfg(steps, checkpoint_every, precision, tau, force, inlet, axis)
        Y, Z = self.params.lb_size[1], self.params.lb_size[2]
        J, dF, dtau, duin = np.zeros(1), np.zeros(3), np.zeros(1), np.zeros(Y * Z)
        check(self.L.hb_adjoint_drag(self.h, C.byref(cfg), _p(J), _p(dF), _p(dtau), _p(duin)))
        return float(J[0]), dF, float(dtau[0]), duin

    def adjoint_timing(self):
        f, r, nf, nr = C.c_float(0), C.c_float(0), C.c_int64(0), C.c_int64(0)
        check(self.L.hb_adjoint_timing(self.h, C.byref(f), C.byref(r), C.byref(nf), C.byref(nr)))
        return f.value, r.value, nf.value, nr.value
