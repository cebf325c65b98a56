"""Synthetic workloads with the shapes of the benchmark configurations (seeded; no data
files).  Each returns hb_params plus the particle / object arrays the C-ABI takes."""
import numpy as np

from . import abi


def channel(shape=(64, 32, 32), precision=abi.HB_FP64, collision=abi.HB_BGK, tau=0.8, force=1e-6,
            magic=3.0 / 16.0):
    """Periodic channel, walls at y (boundary codes x 4/4, y 7/7, z 4/4), force along x."""
    return abi.make_params(shape, (4, 4, 7, 7, 4, 4), init_visc=(tau - 0.5) / 3.0, lbF=(force, 0, 0),
                           precision=precision, collision=collision, trt_magic=magic)


def inlet_profile(shape, u0, zwave=0.0):
    """x-velocity of the two x planes, index y + Y*z: a parabola across the channel
    height (zero at the half-way walls y = 0.5 and y = Y - 1.5), optionally modulated
    along z by (1 + zwave sin(2 pi z / Z))."""
    X, Y, Z = shape
    s = np.clip((np.arange(Y) - 0.5) / (Y - 2), 0.0, 1.0)
    prof = u0 * 4.0 * s * (1.0 - s)
    mod = 1.0 + zwave * np.sin(2.0 * np.pi * np.arange(Z) / Z)
    return np.ascontiguousarray((mod[:, None] * prof[None, :]).reshape(-1))


def adjoint_channel(shape=(96, 96, 96), per_axis=4, radius=6.0, jitter=2.0, seed=5, tau=0.7, force=2e-6,
                    u0=0.02, precision=abi.HB_FP32, zwave=0.0):
    """Drag-adjoint workload: a channel with moving-wall inlet/outlet planes at x
    (code 8, velocity u_in(y,z) along x), static walls at y, periodic z, and
    per_axis^3 fixed spheres ("objects") on a jittered lattice of spacing L/per_axis.
    TRT, relaxation time tau, body force along x."""
    X, Y, Z = shape
    rng = np.random.default_rng(seed)
    sp = np.array(shape, dtype=float) / per_axis
    k = np.arange(per_axis) + 0.5
    cent = np.stack(np.meshgrid(k * sp[0], k * sp[1], k * sp[2], indexing="ij"), -1).reshape(-1, 3)
    cent = cent + rng.uniform(-jitter, jitter, size=cent.shape)
    objects = np.c_[cent, np.full(len(cent), radius)]
    params = abi.make_params(shape, (8, 8, 7, 7, 4, 4), init_visc=(tau - 0.5) / 3.0, lbF=(force, 0.0, 0.0),
                             collision=abi.HB_TRT, precision=precision)
    return params, objects, inlet_profile(shape, u0, zwave)
