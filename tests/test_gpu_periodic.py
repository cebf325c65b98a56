"""Periodic faces with moving particles: pbcShift, ghost particles, the reference's
half-shell neighbour sweep over them (DEM.cpp:1395-1494, 1554-1664) and, with the
lattice, the re-mark of the particle nodes after each rebuild (updateIndices,
LB.cpp:1826-1849) -- against fixtures written by the reference itself
(tests/golden/make_golden.py: dem_periodic, box_periodic).

Exact: the ghost list (origin and shift, in the reference's order), the candidate pair
set (the reference's table also holds pairs of two ghosts, which carry no force and are
not kept here), node types, particle flags and the particle index of every particle
node (ghost indices included).  FP64 fields to 1e-11 relative (element sums over a
ghost's nodes are added per particle instead of in node order); DEM trajectories as in
the other DEM fixtures (1e-10 before stiff contacts, 1e-5 after)."""
import numpy as np
import pytest

from hybird_gb300 import abi
from oracle_port import golden_params, load_golden, rel_linf

pytestmark = pytest.mark.gpu


def _gpu():
    from hybird_gb300.gpu import GpuSim
    return GpuSim


def _ref_pairs(d, pre, E):
    rp = np.sort(d[pre + "neighborTable"].reshape(-1, 2).astype(np.int64), axis=1)
    rp = rp[rp[:, 0] < E]  # at least one standard particle
    return rp[np.lexsort((rp[:, 1], rp[:, 0]))]


def _check_ghosts(g, d, pre):
    go, gv = g.ghosts()
    np.testing.assert_array_equal(go, d[pre + "ghost_index"], err_msg=pre)
    np.testing.assert_array_equal(gv, d[pre + "ghost_vec"].reshape(-1, 3), err_msg=pre)


def test_dem_periodic_matches_reference_fixture():
    d = load_golden("dem_periodic")
    p = golden_params(d)
    E = d["spheres"].shape[0]
    g = _gpu()(p, d["spheres"], d["objects"])
    done = 0
    seen_ghost_pairs = 0
    for step in d["steps"]:
        if step > done:
            g.cycle(int(step) - done)
            done = int(step)
        pre = f"s{step}_"
        _check_ghosts(g, d, pre)
        ge = g.elements()
        early = step <= 60
        for k, gk, tol in (("x0", "e_x0", 1e-10 if early else 1e-5), ("x1", "e_x1", 1e-8 if early else 1e-2)):
            ref = d[pre + gk].reshape(-1, 3).T.reshape(-1)
            assert rel_linf(ge[k], ref) <= tol, (step, k, rel_linf(ge[k], ref))
        if step > 0:
            gp = g.pairs().reshape(-1, 2).astype(np.int64)
            rp = _ref_pairs(d, pre, E)
            np.testing.assert_array_equal(gp, rp, err_msg=f"step {step}")
            seen_ghost_pairs += int((gp[:, 1] >= E).sum())
    assert seen_ghost_pairs > 0
    g.close()


@pytest.mark.parametrize("prec", [abi.HB_FP64, abi.HB_FP32])
def test_box_periodic_matches_reference_fixture(prec):
    d = load_golden("box_periodic")
    p = golden_params(d, precision=prec)
    E = d["spheres"].shape[0]
    g = _gpu()(p, d["spheres"], d["objects"])
    done = 0
    ghost_nodes = 0
    for step in d["steps"]:
        if step > done:
            g.cycle(int(step) - done)
            done = int(step)
        pre = f"s{step}_"
        _check_ghosts(g, d, pre)
        gl = g.lattice()
        if prec == abi.HB_FP64 or step <= 10:
            np.testing.assert_array_equal(gl["type"], d[pre + "type"])
            np.testing.assert_array_equal(gl["inside"], d[pre + "inside"], err_msg=f"step {step}")
            inside = d[pre + "inside"] == 1
            np.testing.assert_array_equal(gl["solid"][inside], d[pre + "solid"][inside], err_msg=f"step {step}")
            ghost_nodes += int((d[pre + "solid"][inside] >= E).sum())
        act = (d[pre + "type"] == 0) | (d[pre + "type"] == 3)
        if step == 0:
            continue
        ge = g.elements()
        if prec == abi.HB_FP64:
            assert rel_linf(gl["n"], d[pre + "n"], act) <= 1e-11, (step, "n")
            assert rel_linf(gl["u"].reshape(3, -1), d[pre + "u"].reshape(3, -1), act) <= 1e-11, (step, "u")
            if pre + "f" in d.files:
                assert rel_linf(gl["f"].reshape(19, -1), d[pre + "f"].reshape(19, -1), act) <= 1e-11, (step, "f")
            for k, gk in (("x0", "e_x0"), ("x1", "e_x1"), ("FHydro", "e_FHydro"), ("MHydro", "e_MHydro")):
                ref = d[pre + gk].reshape(-1, 3).T.reshape(-1)
                assert rel_linf(ge[k], ref) <= 1e-10, (step, k, rel_linf(ge[k], ref))
            np.testing.assert_array_equal(g.pairs().reshape(-1, 2).astype(np.int64), _ref_pairs(d, pre, E))
        else:
            du = gl["u"].reshape(3, -1)[:, act] - d[pre + "u"].reshape(3, -1)[:, act]
            l2 = np.sqrt((du ** 2).sum() / (d[pre + "u"].reshape(3, -1)[:, act] ** 2).sum())
            assert l2 <= 1e-4, (step, l2)
            ref = d[pre + "e_x0"].reshape(-1, 3).T.reshape(-1)
            assert rel_linf(ge["x0"], ref) <= 1e-5, (step, rel_linf(ge["x0"], ref))
    assert ghost_nodes > 0
    g.close()


def test_dem_periodic_objects_matches_reference_fixture():
    """Fixed objects near periodic faces get periodic images (DEM::periodicObjects,
    DEM.cpp:990-1063): spheres driven along x through the faces meet an object's image
    across the face.  Against the reference's fixture: the object count with images, the
    ghost list, the candidate pair set, the objects' particle forces and the element
    trajectories (which the image contacts change)."""
    d = load_golden("dem_periodic_objects")
    p = golden_params(d)
    E = d["spheres"].shape[0]
    g = _gpu()(p, d["spheres"], d["objects"])
    n_std = d["objects"].shape[0]
    n_all = d["s0_o_FParticle"].size // 3  # the reference's objects list, images appended
    assert n_all > n_std
    assert len(g.objects()) == 3 * n_all
    image_hits = 0
    done = 0
    for step in d["steps"]:
        if step > done:
            g.cycle(int(step) - done)
            done = int(step)
        pre = f"s{step}_"
        _check_ghosts(g, d, pre)
        near = d[pre + "nearObjectTable"].reshape(-1, 2)
        image_hits += int((near[:, 1] >= n_std).sum())
        ge = g.elements()
        early = step <= 60
        for k, gk, tol in (("x0", "e_x0", 1e-10 if early else 1e-5), ("x1", "e_x1", 1e-8 if early else 1e-2)):
            ref = d[pre + gk].reshape(-1, 3).T.reshape(-1)
            assert rel_linf(ge[k], ref) <= tol, (step, k, rel_linf(ge[k], ref))
        if step > 0:
            np.testing.assert_array_equal(g.pairs().reshape(-1, 2).astype(np.int64), _ref_pairs(d, pre, E),
                                          err_msg=f"step {step}")
        ref_o = d[pre + "o_FParticle"]
        go = g.objects()
        assert np.abs(go - ref_o).max() <= 1e-10 * max(1.0, np.abs(ref_o).max()), (step, go, ref_o)
    assert image_hits > 0  # some sphere had an object image in range
    g.close()
