"""Synthetic workloads with the shapes of the benchmark configurations (seeded; no data
files).  Each returns hb_params plus the particle / object arrays the C-ABI takes."""
import numpy as np

from . import abi


def channel(shape=(64, 32, 32), precision=abi.HB_FP64, collision=abi.HB_BGK, tau=0.8, force=1e-6,
            magic=3.0 / 16.0):
    """Periodic channel, walls at y (boundary codes x 4/4, y 7/7, z 4/4), force along x."""
    return abi.make_params(shape, (4, 4, 7, 7, 4, 4), init_visc=(tau - 0.5) / 3.0, lbF=(force, 0, 0),
                           precision=precision, collision=collision, trt_magic=magic)


def rsa_spheres(seed, n, rmin, rmax, lo, hi, attempts=2_000_000):
    """Random sequential addition of non-overlapping spheres, radius U[rmin, rmax], centres
    in [lo + r, hi - r] per axis (lo, hi scalars or 3-vectors).  Stops at n spheres or
    after `attempts` tries.  A cell list keeps each test local."""
    rng = np.random.default_rng(seed)
    lo = np.broadcast_to(np.asarray(lo, dtype=float), (3,))
    hi = np.broadcast_to(np.asarray(hi, dtype=float), (3,))
    cw = 2.0 * rmax
    cells = {}
    out = []
    tries = 0
    while len(out) < n and tries < attempts:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = lo + r + rng.random(3) * (hi - lo - 2 * r)
        key = tuple((c // cw).astype(int))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for s in cells.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                        if (c[0] - s[0]) ** 2 + (c[1] - s[1]) ** 2 + (c[2] - s[2]) ** 2 < (r + s[3]) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            s = (c[0], c[1], c[2], r)
            out.append(s)
            cells.setdefault(key, []).append(s)
    return np.array(out).reshape(-1, 4)


def precision_box(precision, n=16000, L=256, seed=4):
    """Configuration 4: the coupled sedimentation box at L^3 with n spheres r ~ U[3, 5]
    (seeded RSA), TRT tau 0.8, gravity 1e-5, linear contacts, multiStep 3."""
    spheres = rsa_spheres(seed, n, 3.0, 5.0, 0.5, L - 1.5)
    p = abi.make_params((L, L, L), (7,) * 6, init_visc=(0.8 - 0.5) / 3.0, lbF=(0.0, 0.0, -1e-5),
                        collision=abi.HB_TRT, precision=precision, multi_step=3, density=2.5,
                        linear_stiff=1e3, restitution=0.8, friction_part=0.5, friction_wall=0.5, visc_tang=0.5)
    return p, spheres


def dam_break(precision, shape=(256, 128, 128), n=500, seed=6, yield_stress=None):
    """Configuration 3: free-surface dam break, liquid column x < 0.4 X, z < 0.6 Z, Bingham
    plastic (plastic viscosity for tau 0.6, yield stress U[1e-6, 1e-5] drawn once per seed)
    with Smagorinsky (turbConst 0.01, Cs = 0.1), gravity 1e-5 along -z, n spheres r = 5
    seeded in the column, walls on all faces."""
    X, Y, Z = shape
    rng = np.random.default_rng(seed)
    ys = rng.uniform(1e-6, 1e-5) if yield_stress is None else yield_stress
    spheres = rsa_spheres(seed, n, 5.0, 5.0, (0.5, 0.5, 0.5), (0.4 * X - 1.0, Y - 1.5, 0.6 * Z - 1.0))
    p = abi.make_params(shape, (7,) * 6, init_visc=(0.6 - 0.5) / 3.0, lbF=(0.0, 0.0, -1e-5),
                        non_newtonian=1, plastic_visc=(0.6 - 0.5) / 3.0, yield_stress=ys, turbulence=1,
                        turb_const=0.01, free_surface=1, gas_box=(0.4, 0.6), collision=abi.HB_BGK,
                        precision=precision, multi_step=3, density=2.5)
    return p, spheres


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
