"""hb_download_elements_async: the element state of every step, queued behind the step
without a host wait, equals the synchronous download's -- into page-locked mapped arrays
(written by the gather kernel itself) and into plain pageable arrays (copies)."""
import ctypes as C

import numpy as np
import pytest

from hybird_gb300 import abi

pytestmark = pytest.mark.gpu


def _sim():
    from hybird_gb300.gpu import GpuSim
    spheres = np.array([[7.3, 6.6, 8.1, 2.6], [12.2, 11.7, 9.4, 2.9], [8.0, 13.0, 13.5, 2.2]])
    p = abi.make_params((20, 18, 20), (7,) * 6, init_visc=0.1, lbF=(0.0, 0.0, -2e-4), multi_step=3,
                        precision=abi.HB_FP32)
    return GpuSim(p, spheres)


@pytest.mark.parametrize("mapped", [True, False])
def test_async_element_download_matches_sync(mapped):
    from hybird_gb300.gpu import check
    g = _sim()
    L = g.L
    E = g.E
    steps = 6
    host = np.full((steps, 4, 3 * E), np.nan)
    if mapped:
        check(L.hb_host_register(host.ctypes.data_as(C.c_void_p), host.nbytes))
    ref = []
    g2 = _sim()
    for s in range(steps):
        check(L.hb_cycle(g.h, 1))
        ptr = [host[s, k].ctypes.data_as(C.c_void_p) for k in range(4)]
        check(L.hb_download_elements_async(g.h, ptr[0], ptr[1], None, None, ptr[2], ptr[3],
                                           None, None, None, None, None))
        g2.cycle(1)
        e = g2.elements()
        ref.append(np.stack([e["x0"], e["x1"], e["FHydro"], e["MHydro"]]))
    check(L.hb_synchronize(g.h))
    if mapped:
        check(L.hb_host_unregister(host.ctypes.data_as(C.c_void_p)))
    for s in range(steps):
        np.testing.assert_array_equal(host[s], ref[s], err_msg=f"step {s}")
    assert np.abs(host[-1, 2]).max() > 0.0
    g.close()
    g2.close()
