"""The allocation-free entry point hb_wall_force_noalloc.

It exists for callers that cannot call cudaMalloc (an application whose own pool
allocator owns the device memory and gives this library a fixed budget, or a host loop
that cannot take the device-wide synchronisation of an allocation): it computes the
moving-wall momentum exchange from caller device buffers with its scratch in a fixed
device array inside the library.  This test runs a channel with a moving wall through
the regular context, then hands the same streamed state to the allocation-free entry
point twice in a row and checks both results against the context's own wall forces
(hb_download_walls) and the extra mass against a numpy restatement of the moving-wall
rule (LB.cpp:1321-1341), to FP64 rounding.

Named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from hybird_gb300 import abi

pytestmark = pytest.mark.gpu


# D3Q19 in the reference's order (lattice.h:36-60)
C_X = [1 if j in (1, 7, 10, 15, 17) else -1 if j in (2, 8, 9, 16, 18) else 0 for j in range(19)]
C_Y = [1 if j in (3, 7, 9, 11, 14) else -1 if j in (4, 8, 10, 12, 13) else 0 for j in range(19)]
C_Z = [1 if j in (5, 11, 13, 15, 18) else -1 if j in (6, 12, 14, 16, 17) else 0 for j in range(19)]
W = [12 / 36] + [2 / 36] * 6 + [1 / 36] * 12


def _wall_terms(st, u, size, bnd):
    """numpy restatement of the moving-wall rule (LB.cpp:1321-1341) on a streamed state:
    per wall (solid index of the wall node) the momentum exchange sum of
    (2 (fs_j - w_j) - BBi) c_j with fs_j = f_out[opp j] + BBi, BBi = 6 n w_j (u_wall . c_j),
    and the extra mass sum of BBi * mass, over active nodes and links onto moving walls
    (code 8), links remapped across periodic faces.  Returns the 19 outputs and the sum
    of the absolute extra-mass terms."""
    X, Y, Z = (int(v) for v in size)
    per = [b == 4 for b in bnd]
    N = X * Y * Z
    t = st["type"].reshape(Z, Y, X) & 0x0F
    n, mass = st["n"].reshape(Z, Y, X), st["mass"].reshape(Z, Y, X)
    solid = st["solid"].reshape(Z, Y, X)
    uu = u.reshape(3, Z, Y, X)
    f = st["f"].reshape(19, Z, Y, X)
    z, y, x = np.meshgrid(np.arange(1, Z - 1), np.arange(1, Y - 1), np.arange(1, X - 1), indexing="ij")
    act = (t[z, y, x] == 0) | (t[z, y, x] == 3)
    out = np.zeros(19)
    terms = 0.0
    for j in range(1, 19):
        o = j + 1 if j % 2 else j - 1
        xn, yn, zn = x + C_X[j], y + C_Y[j], z + C_Z[j]
        for a, dim, lo, hi in ((xn, X, per[0], per[1]), (yn, Y, per[2], per[3]), (zn, Z, per[4], per[5])):
            a[(a == 0) & lo] = dim - 2
            a[(a == dim - 1) & hi] = 1
        hit = act & (t[zn, yn, xn] == 8)
        uw = uu[0][zn, yn, xn] * C_X[j] + uu[1][zn, yn, xn] * C_Y[j] + uu[2][zn, yn, xn] * C_Z[j]
        bbi = 6.0 * n[z, y, x] * W[j] * uw
        fs = f[o][z, y, x] + bbi
        sc = (2.0 * (fs - W[j]) - bbi)[hit]
        wi = solid[zn, yn, xn][hit]
        for k, c in enumerate((C_X[j], C_Y[j], C_Z[j])):
            np.add.at(out, 3 * wi + k, sc * c)
        v = (bbi * mass[z, y, x])[hit]
        out[18] += v.sum()
        terms += np.abs(v).sum()
    return out, terms


def test_wall_force_noalloc_matches_context_twice():
    torch = pytest.importorskip("torch")
    from hybird_gb300.gpu import GpuSim, lib

    p = abi.make_params((20, 12, 10), (4, 4, 7, 8, 4, 4), init_visc=0.05, lbF=(2e-5, 0.0, -1e-5),
                        init_velocity=(0.02, 0.0, 0.01), precision=abi.HB_FP64)
    g = GpuSim(p)
    g.cycle(7)
    ref, _ = g.walls()
    st = g.lattice()
    assert np.abs(ref).max() > 0.0
    L = lib()
    L.hb_wall_force_noalloc.argtypes = [C.c_void_p] * 8 + [C.c_void_p, C.c_void_p]
    L.hb_wall_force_noalloc.restype = C.c_int
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(st[k])).to(dev) for k in ("f", "type", "solid", "n", "u", "mass")}
    size = np.array(p.lb_size[:], dtype=np.int32)
    bnd = np.array(p.boundary[:], dtype=np.int32)
    results = []
    for _ in range(2):
        out = torch.full((19,), float("nan"), dtype=torch.float64, device=dev)
        rc = L.hb_wall_force_noalloc(t["f"].data_ptr(), t["type"].data_ptr(), t["solid"].data_ptr(),
                                     t["n"].data_ptr(), t["u"].data_ptr(), t["mass"].data_ptr(),
                                     size.ctypes.data, bnd.ctypes.data, out.data_ptr(), None)
        assert rc == abi.HB_OK
        torch.cuda.synchronize()
        results.append(out.cpu().numpy())
    nw = len(ref) // 3
    scale = np.abs(ref).max()
    for res in results:
        assert np.all(np.isfinite(res))
        assert np.abs(res[:3 * nw] - ref).max() <= 1e-12 * scale, (res[:3 * nw], ref)
    assert np.array_equal(results[0], results[1])
    # walls from boundary codes do not move (DEM.cpp:452-457), so the extra mass above is
    # zero; a third call with a velocity on the moving-wall nodes checks the extra-mass
    # output and the wall forces against the numpy restatement
    u2 = st["u"].reshape(3, -1).copy()
    wall = (st["type"] & 0x0F) == 8
    # a normal component: for a purely tangential wall velocity the extra-mass terms of
    # each node cancel over its links
    u2[0, wall], u2[1, wall], u2[2, wall] = 0.01, -0.003, 0.002
    u2 = np.ascontiguousarray(u2.reshape(-1))
    t["u"] = torch.from_numpy(u2).to(dev)
    out = torch.full((19,), float("nan"), dtype=torch.float64, device=dev)
    rc = L.hb_wall_force_noalloc(t["f"].data_ptr(), t["type"].data_ptr(), t["solid"].data_ptr(),
                                 t["n"].data_ptr(), t["u"].data_ptr(), t["mass"].data_ptr(),
                                 size.ctypes.data, bnd.ctypes.data, out.data_ptr(), None)
    assert rc == abi.HB_OK
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    want, terms = _wall_terms(st, u2, size, bnd)
    assert terms > 0.0
    assert abs(res[18] - want[18]) <= 1e-12 * terms, (res[18], want[18])
    assert np.abs(res[:18] - want[:18]).max() <= 1e-12 * np.abs(want[:18]).max(), (res[:18], want[:18])
    g.close()


def test_wall_force_noalloc_rejects_oversize_lattice():
    from hybird_gb300.gpu import lib

    L = lib()
    L.hb_wall_force_noalloc.argtypes = [C.c_void_p] * 8 + [C.c_void_p, C.c_void_p]
    size = np.array([1 << 10, 1 << 10, 1 << 9], dtype=np.int32)  # 2^29 nodes > 2^28
    bnd = np.array([7] * 6, dtype=np.int32)
    dummy = C.c_void_p(1)
    rc = L.hb_wall_force_noalloc(dummy, dummy, dummy, dummy, dummy, dummy, size.ctypes.data,
                                 bnd.ctypes.data, dummy, None)
    assert rc == 1  # HB_ERR_ARG, before any device access
