"""Synthetic workloads with the shapes of the benchmark configurations (seeded; no data
files).  Each returns hb_params plus the particle / object arrays the C-ABI takes."""
import functools

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


def deposit(spheres, floor=0.5, overlap=1e-4):
    """The same spheres dropped straight down, lowest first, onto the floor plane z =
    floor (the no-slip wall of the lower z face, DEM.cpp:435-633) or onto a sphere
    already resting, and left there pressed in by `overlap` (near the static overlap of
    a linear spring under a sphere's weight).  x and y stay as given, so a packing that
    does not overlap in the plane keeps every sphere inside the box; the result is a bed
    in which every sphere touches the floor or another sphere from the first substep
    on.  Overlaps with spheres other than the one a sphere lands on stay below
    `overlap`."""
    s = np.asarray(spheres, dtype=float)
    out = s.copy()
    placed = []
    for k in np.argsort(s[:, 2], kind="stable"):
        x, y, r = s[k, 0], s[k, 1], s[k, 3]
        z = floor + r - overlap
        if placed:
            q = out[placed]
            h2 = (q[:, 0] - x) ** 2 + (q[:, 1] - y) ** 2
            reach = (q[:, 3] + r) ** 2 - h2
            hit = reach > 0.0
            if hit.any():
                z = max(z, float((q[hit, 2] + np.sqrt(reach[hit])).max()) - overlap)
        out[k, 2] = z
        placed.append(k)
    return out


def sedimentation(precision, L=128, seed=2, collision=None, deposited=False):
    """Configuration 2: coupled sedimentation in an L^3 no-slip box, seeded random
    sequential addition of spheres r ~ U[4, 6] until it jams (about 1500 at L = 128),
    density ratio 2.5, gravity 1e-5 along -z, linear contacts kn = 1e3, e = 0.8,
    mu = 0.5, viscTang 0.5, multiStep 3, TRT tau 0.8 (BGK with collision=HB_BGK).
    deposited=True drops the same spheres onto the floor first (deposit), so that the
    contact path runs from the first substep, and takes multiStep 10: in a bed where a
    sphere touches several neighbours the Gear predictor-corrector (elmt.cpp:139-254) is
    unstable at multiStep 3 and 6 (the oracle's particle speeds grow about 2.3-fold per
    cycle at 3) and stable at 10."""
    spheres = _rsa_cached(seed, 2000, 4.0, 6.0, 0.5, L - 1.5).copy()
    if deposited:
        spheres = deposit(spheres)
    p = abi.make_params((L, L, L), (7,) * 6, init_visc=(0.8 - 0.5) / 3.0, lbF=(0.0, 0.0, -1e-5),
                        collision=abi.HB_TRT if collision is None else collision, trt_magic=3.0 / 16.0,
                        precision=precision, multi_step=10 if deposited else 3, density=2.5, linear_stiff=1e3,
                        restitution=0.8,
                        friction_part=0.5, friction_wall=0.5, visc_tang=0.5)
    return p, spheres


@functools.lru_cache(maxsize=8)
def _rsa_cached(seed, target, rmin, rmax, lo, hi):
    return _rsa_batched(seed, target, rmin, rmax, lo, hi)


def _rsa_batched(seed, target, rmin, rmax, lo, hi, tries=400000, batch=4096):
    """Seeded random sequential addition of non-overlapping spheres, drawn in batches of
    `batch` candidates (radius, then x, y, z centres); a candidate is accepted when it
    overlaps no sphere placed before it, earlier accepted candidates of its own batch
    included.  Stops at `target` spheres or after `tries` candidates.  Placed spheres are
    binned in cells of width 2 rmax, so each test looks at the 27 cells around the
    candidate only (the same acceptance as testing every placed sphere)."""
    rng = np.random.default_rng(seed)
    cw = 2.0 * rmax
    ncell = int(np.ceil((hi - lo) / cw)) + 1
    cap = 8  # non-overlapping spheres of radius >= rmin / 2 per cell of width 2 rmax
    grid = np.full((ncell, ncell, ncell, cap), -1, dtype=np.int64)
    fill = np.zeros((ncell, ncell, ncell), dtype=np.int64)
    placed = np.zeros((target, 4))
    n = 0
    done = 0
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    while done < tries and n < target:
        r = rng.uniform(rmin, rmax, batch)
        c = np.stack([rng.uniform(lo + r, hi - r) for _ in range(3)], axis=1)
        done += batch
        cell = np.clip(((c - lo) // cw).astype(np.int64), 0, ncell - 1)
        nb = np.clip(cell[:, None, :] + offs[None, :, :], 0, ncell - 1)  # clipped repeats are harmless
        idx = grid[nb[..., 0], nb[..., 1], nb[..., 2]].reshape(batch, -1)  # [batch, 27*cap]
        valid = idx >= 0
        q = placed[np.where(valid, idx, 0)]
        d2 = ((c[:, None, :] - q[..., :3]) ** 2).sum(-1)
        ok = ~((d2 < (r[:, None] + q[..., 3]) ** 2) & valid).any(axis=1)
        acc = []
        for k in np.nonzero(ok)[0]:
            good = True
            for a in acc:
                if ((c[k] - c[a]) ** 2).sum() < (r[k] + r[a]) ** 2:
                    good = False
                    break
            if good:
                acc.append(k)
                if n + len(acc) >= target:
                    break
        for k in acc:
            placed[n] = (c[k, 0], c[k, 1], c[k, 2], r[k])
            gx, gy, gz = cell[k]
            grid[gx, gy, gz, fill[gx, gy, gz]] = n
            fill[gx, gy, gz] += 1
            n += 1
    return placed[:n].copy()
