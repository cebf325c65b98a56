"""Multi-sphere elements (DEM::compositeProperties and the element/particle updates,
DEM.cpp:404-433, 1114-1182; elmt.cpp:17-137, 261-290): clusters of 1 to 4 spheres at
the prototype positions, rotated with the element; the contacts act through each
sphere (normal forces with a moment, lever arms with radiusVec); the quaternion
follows q2 = 0.5 qp0 quatAcc(waBf, qp1).  Against fixtures written by the reference
itself (tests/golden/make_golden.py: dem_clusters, box_clusters -- the second also
with periodic x, so ghosts of cluster spheres).

Exact: the candidate pair set over particles (pairs of two ghosts are not kept), the
ghost list, node types, particle flags and particle indices of the particle nodes.
FP64 fields and element states to 1e-10 before the stiff contacts; DEM trajectories
after them as in the other DEM fixtures."""
import numpy as np
import pytest

from hybird_gb300 import abi
from oracle_port import golden_params, load_golden, rel_linf

pytestmark = pytest.mark.gpu


def _sim(d, p):
    from hybird_gb300.gpu import GpuSim
    return GpuSim(p, d["spheres"], d["objects"], sizes=d["sizes"], quats=d["quats"])


def _ref_pairs(d, pre, P):
    rp = np.sort(d[pre + "neighborTable"].reshape(-1, 2).astype(np.int64), axis=1)
    rp = rp[rp[:, 0] < P]
    return rp[np.lexsort((rp[:, 1], rp[:, 0]))]


def _elements_close(g, d, pre, tol_x, tol_v):
    ge = g.elements()
    for k, gk, tol in (("x0", "e_x0", tol_x), ("x1", "e_x1", tol_v), ("w", "e_w", tol_v)):
        ref = d[pre + gk].reshape(-1, 3).T.reshape(-1)
        if np.abs(ref).max() == 0.0:
            assert np.abs(ge[k]).max() == 0.0, (pre, k)
            continue
        assert rel_linf(ge[k], ref) <= tol, (pre, k, rel_linf(ge[k], ref))
    qref = d[pre + "e_q0"].reshape(-1, 4).T.reshape(-1)
    assert np.abs(ge["q0"] - qref).max() <= tol_v, (pre, "q0", np.abs(ge["q0"] - qref).max())


def test_dem_clusters_match_reference_fixture():
    d = load_golden("dem_clusters")
    p = golden_params(d)
    P = int(d["sizes"].sum())
    g = _sim(d, p)
    done = 0
    for step in d["steps"]:
        if step > done:
            g.cycle(int(step) - done)
            done = int(step)
        pre = f"s{step}_"
        early = step <= 100
        _elements_close(g, d, pre, 1e-10 if early else 1e-5, 1e-8 if early else 1e-2)
        if step > 0:
            np.testing.assert_array_equal(g.pairs().reshape(-1, 2).astype(np.int64), _ref_pairs(d, pre, P),
                                          err_msg=f"step {step}")
    g.close()


@pytest.mark.parametrize("prec", [abi.HB_FP64, abi.HB_FP32])
def test_box_clusters_match_reference_fixture(prec):
    d = load_golden("box_clusters")
    p = golden_params(d, precision=prec)
    P = int(d["sizes"].sum())
    g = _sim(d, p)
    done = 0
    for step in d["steps"]:
        if step > done:
            g.cycle(int(step) - done)
            done = int(step)
        pre = f"s{step}_"
        go, gv = g.ghosts()
        np.testing.assert_array_equal(go, d[pre + "ghost_index"], err_msg=pre)
        np.testing.assert_array_equal(gv, d[pre + "ghost_vec"].reshape(-1, 3), err_msg=pre)
        gl = g.lattice()
        if prec == abi.HB_FP64 or step <= 10:
            np.testing.assert_array_equal(gl["type"], d[pre + "type"])
            np.testing.assert_array_equal(gl["inside"], d[pre + "inside"], err_msg=f"step {step}")
            inside = d[pre + "inside"] == 1
            np.testing.assert_array_equal(gl["solid"][inside], d[pre + "solid"][inside], err_msg=f"step {step}")
        if step == 0:
            continue
        act = (d[pre + "type"] == 0) | (d[pre + "type"] == 3)
        if prec == abi.HB_FP64:
            assert rel_linf(gl["n"], d[pre + "n"], act) <= 1e-11, (step, "n")
            assert rel_linf(gl["u"].reshape(3, -1), d[pre + "u"].reshape(3, -1), act) <= 1e-11, (step, "u")
            if pre + "f" in d.files:
                assert rel_linf(gl["f"].reshape(19, -1), d[pre + "f"].reshape(19, -1), act) <= 1e-11, (step, "f")
            _elements_close(g, d, pre, 1e-10, 1e-8)
            ge = g.elements()
            for k, gk in (("FHydro", "e_FHydro"), ("MHydro", "e_MHydro")):
                ref = d[pre + gk].reshape(-1, 3).T.reshape(-1)
                assert rel_linf(ge[k], ref) <= 1e-9, (step, k, rel_linf(ge[k], ref))
            np.testing.assert_array_equal(g.pairs().reshape(-1, 2).astype(np.int64), _ref_pairs(d, pre, P))
        else:
            du = gl["u"].reshape(3, -1)[:, act] - d[pre + "u"].reshape(3, -1)[:, act]
            l2 = np.sqrt((du ** 2).sum() / (d[pre + "u"].reshape(3, -1)[:, act] ** 2).sum())
            assert l2 <= 1e-4, (step, l2)
            _elements_close(g, d, pre, 1e-5, 1e-2)
    g.close()
