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


@pytest.mark.parametrize("prec", [abi.HB_FP32, abi.HB_FP64])
def test_element_sink_matches_download(prec):
    """hb_set_element_sink: the cycle graphs write the element state into the registered
    arrays at the end of every cycle; after each step it equals a second context's
    download bit for bit, and removing the sink leaves the arrays alone."""
    from hybird_gb300.gpu import GpuSim, check
    spheres = np.array([[7.3, 6.6, 8.1, 2.6], [12.2, 11.7, 9.4, 2.9], [8.0, 13.0, 13.5, 2.2]])
    p = abi.make_params((20, 18, 20), (7,) * 6, init_visc=0.1, lbF=(0.0, 0.0, -2e-4), multi_step=3,
                        precision=prec)
    g, g2 = GpuSim(p, spheres), GpuSim(p, spheres)
    L, E = g.L, g.E
    host = np.full((4, 3 * E), np.nan)
    vp = host.ctypes.data_as(C.c_void_p)
    check(L.hb_host_register(vp, host.nbytes))
    ptr = [host[k].ctypes.data_as(C.c_void_p) for k in range(4)]
    check(L.hb_set_element_sink(g.h, ptr[0], ptr[1], None, None, ptr[2], ptr[3], None, None, None, None, None))
    for s in range(5):
        check(L.hb_cycle(g.h, 1))
        check(L.hb_synchronize(g.h))
        g2.cycle(1)
        e = g2.elements()
        np.testing.assert_array_equal(host, np.stack([e["x0"], e["x1"], e["FHydro"], e["MHydro"]]),
                                      err_msg=f"step {s}")
    assert np.abs(host[2]).max() > 0.0
    check(L.hb_set_element_sink(g.h, *([None] * 11)))
    before = host.copy()
    g.cycle(2)
    np.testing.assert_array_equal(host, before)
    check(L.hb_host_unregister(vp))
    g.close()
    g2.close()


@pytest.mark.parametrize("spheres", [True, False])
def test_body_force_change_matches_oracle(spheres):
    """hb_set_body_force between cycles (with particles the value rides in the cycle
    graphs' mask kernel parameters; without, a launch of its own) against the oracle
    changing lb.lbF at the same steps: FP64 to 1e-12."""
    from oracle_port import OracleSim, rel_linf
    from hybird_gb300.gpu import GpuSim, check
    sph = np.array([[7.3, 6.6, 8.1, 2.6], [12.2, 11.7, 9.4, 2.9]]) if spheres else None
    p = abi.make_params((20, 18, 20), (7,) * 6, init_visc=0.1, lbF=(0.0, 0.0, -2e-4), multi_step=3,
                        precision=abi.HB_FP64)
    g, o = GpuSim(p, sph), OracleSim(p, sph)
    forces = [(0.0, 0.0, -2e-4), (1e-4, 0.0, -1e-4), (0.0, -3e-4, 0.0)]
    for F in forces:
        f = np.array(F)
        check(g.L.hb_set_body_force(g.h, f.ctypes.data_as(C.c_void_p)))
        o.set_body_force(f)
        g.cycle(3)
        o.cycle(3)
    lg, lo = g.lattice(), o.lattice()
    np.testing.assert_array_equal(lg["inside"], lo["inside"])
    act = (lo["type"] == 0) | (lo["type"] == 3)
    assert rel_linf(lg["f"].reshape(19, -1), lo["f"].reshape(19, -1), act) <= 1e-12
    assert rel_linf(lg["u"].reshape(3, -1), lo["u"].reshape(3, -1), act) <= 1e-12
    if spheres:
        eg, eo = g.elements(), o.elements()
        assert rel_linf(eg["x0"], eo["x0"]) <= 1e-12
        assert rel_linf(eg["FHydro"], eo["FHydro"]) <= 1e-10
    g.close()
    o.close()


def test_lattice_mirror_off_keeps_the_state_and_guards_the_node_fields():
    """hb_set_lattice_mirror(ctx, 0): the cycles skip writing every node's rho, u and
    hydroForce; the populations, node types and element state stay bit-identical to a
    mirrored run, the node-field downloads report HB_ERR_STATE until a mirrored cycle has
    run, and then equal the mirrored run's."""
    from hybird_gb300.gpu import HbError, check
    a, b = _sim(), _sim()
    check(a.L.hb_set_lattice_mirror(a.h, 0))
    a.cycle(5)
    b.cycle(5)
    la, lb = a.lattice(("type", "f")), b.lattice(("type", "f"))
    np.testing.assert_array_equal(la["type"], lb["type"])
    np.testing.assert_array_equal(la["f"], lb["f"])
    ea, eb = a.elements(), b.elements()
    for k in ("x0", "x1", "FHydro", "MHydro"):
        np.testing.assert_array_equal(ea[k], eb[k], err_msg=k)
    with pytest.raises(HbError):
        a.lattice(("n", "u"))
    with pytest.raises(HbError):
        a.export_values()
    check(a.L.hb_set_lattice_mirror(a.h, 1))
    a.cycle(1)
    b.cycle(1)
    la, lb = a.lattice(("n", "u", "hydroForce")), b.lattice(("n", "u", "hydroForce"))
    for k in ("n", "u", "hydroForce"):
        np.testing.assert_array_equal(la[k], lb[k], err_msg=k)
    a.close()
    b.close()
