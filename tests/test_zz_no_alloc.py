"""The allocation-free entry point hb_wall_force_noalloc.

It exists for callers that cannot call cudaMalloc (a host driver that captures every
solver step into a CUDA graph, or an integration held to a fixed device-memory budget):
it computes the moving-wall momentum exchange from caller device buffers with its
scratch in a fixed device array inside the library.  This test runs a channel with a
moving wall through the regular context, then hands the same streamed state to the
allocation-free entry point twice in a row and checks both results against the
context's own wall forces (hb_download_walls), to FP64 rounding.

Named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from hybird_gb300 import abi

pytestmark = pytest.mark.gpu


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
