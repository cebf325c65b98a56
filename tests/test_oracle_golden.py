"""Pins the CPU oracle (oracle/hb_oracle.cpp) to the reference itself: every fixture in
tests/golden/ was produced by the unmodified reference sources (make_golden.py).

Single-phase, coupled and free-surface lattice fields must match the reference
bit-for-bit or to FP64 rounding (1e-13 relative); integer artefacts (node types,
particle flags, solid indices, interface sets, DEM pair sets) must be identical.
"""
import numpy as np
import pytest

from oracle_port import golden_cylinders, OracleSim, golden_gasbox, golden_params, load_golden, rel_linf

LATTICE_CASES = ["channel_bgk", "channel_movwall", "channel_bingham_smag", "box_spheres",
                 "dambreak_fs", "channel_slip", "box_slip", "dambreak_slip", "pipe_curved", "pipe_spheres"]
TOL = 1e-13


def _run(name):
    d = load_golden(name)
    p = golden_params(d, gas_box=golden_gasbox(name))
    sim = OracleSim(p, d["spheres"], d["objects"], cylinders=golden_cylinders(d))
    return d, sim


@pytest.mark.parametrize("name", LATTICE_CASES)
def test_lattice_matches_reference(name):
    d, sim = _run(name)
    done = 0
    for step in d["steps"]:
        sim.cycle(int(step) - done)
        done = int(step)
        g = {k[len(f"s{step}_"):]: d[k] for k in d.files if k.startswith(f"s{step}_")}
        o = sim.lattice()
        np.testing.assert_array_equal(o["type"], g["type"], err_msg=f"{name} step {step} type")
        np.testing.assert_array_equal(o["inside"], g["inside"], err_msg=f"{name} step {step} inside")
        act = (g["type"] == 0) | (g["type"] == 3)
        np.testing.assert_array_equal(o["solid"][act | (g["type"] >= 7)], g["solid"][act | (g["type"] >= 7)])
        assert rel_linf(o["n"], g["n"], act) <= TOL, (name, step, "n")
        assert rel_linf(o["u"].reshape(3, -1), g["u"].reshape(3, -1), act) <= TOL, (name, step, "u")
        assert rel_linf(o["mass"], g["mass"], act) <= TOL, (name, step, "mass")
        assert rel_linf(o["visc"], g["visc"], act) <= TOL, (name, step, "visc")
        if "f" in g:
            assert rel_linf(o["f"].reshape(19, -1), g["f"].reshape(19, -1), act) <= TOL, (name, step, "f")
            assert rel_linf(o["hydroForce"].reshape(3, -1), g["hydroForce"].reshape(3, -1), act) <= TOL or \
                np.abs(g["hydroForce"]).max() == 0.0
        np.testing.assert_array_equal(np.sort(sim.interface()), np.sort(g["interfaceNodes"]))
        fh, _ = sim.walls()
        if len(g["w_FHydro"]):
            assert np.allclose(fh, g["w_FHydro"], rtol=1e-12, atol=1e-15), (name, step, fh, g["w_FHydro"])


@pytest.mark.parametrize("name", ["box_spheres", "dem_objects", "dem_hertz", "dem_cylinder", "pipe_spheres"])
def test_dem_matches_reference(name):
    d, sim = _run(name)
    done = 0
    for step in d["steps"]:
        sim.cycle(int(step) - done)
        done = int(step)
        pre = f"s{step}_"
        e = sim.elements()
        for k, gk in (("x0", "e_x0"), ("x1", "e_x1"), ("w", "e_w"), ("FHydro", "e_FHydro"),
                      ("MHydro", "e_MHydro"), ("FParticle", "e_FParticle"), ("FWall", "e_FWall")):
            g = d[pre + gk].reshape(-1, 3).T.reshape(-1)
            if np.abs(g).max() == 0:
                assert np.abs(e[k]).max() == 0, (name, step, k)
            else:
                assert rel_linf(e[k], g) <= 1e-12, (name, step, k, rel_linf(e[k], g))
        pairs = sim.pairs().reshape(-1, 2)
        gp = d[pre + "neighborTable"].reshape(-1, 2)
        np.testing.assert_array_equal(pairs, gp)  # same sweep order as the reference


@pytest.mark.parametrize("name", ["dem_periodic", "box_periodic", "dem_clusters", "box_clusters", "dem_periodic_objects"])
def test_periodic_and_cluster_dem_match_reference(name):
    """Ghost particles across periodic faces and multi-sphere elements (DEM.cpp:404-433,
    1395-1494, 1554-1664; LB.cpp:1826-1849): the oracle's candidate table equals the
    reference's in content and order, node flags and particle indices are identical, and
    fields and element states agree to FP64 rounding before stiff contacts."""
    d = load_golden(name)
    p = golden_params(d)
    extra = dict(sizes=d["sizes"], quats=d["quats"]) if "sizes" in d.files else {}
    sim = OracleSim(p, d["spheres"], d["objects"], **extra)
    lattice = p.lb_solve == 1
    done = 0
    for step in d["steps"]:
        sim.cycle(int(step) - done)
        done = int(step)
        pre = f"s{step}_"
        late = name.startswith("dem_") and step > 100
        e = sim.elements()
        for k, gk in (("x0", "e_x0"), ("x1", "e_x1"), ("w", "e_w")):
            g = d[pre + gk].reshape(-1, 3).T.reshape(-1)
            if np.abs(g).max() == 0:
                assert np.abs(e[k]).max() == 0, (name, step, k)
            else:
                assert rel_linf(e[k], g) <= (1e-5 if late else 1e-11), (name, step, k, rel_linf(e[k], g))
        if not late:
            np.testing.assert_array_equal(sim.pairs().reshape(-1, 2), d[pre + "neighborTable"].reshape(-1, 2))
        if lattice:
            o = sim.lattice()
            np.testing.assert_array_equal(o["type"], d[pre + "type"])
            np.testing.assert_array_equal(o["inside"], d[pre + "inside"], err_msg=f"{name} step {step}")
            ins = d[pre + "inside"] == 1
            np.testing.assert_array_equal(o["solid"][ins], d[pre + "solid"][ins])
            act = (d[pre + "type"] == 0) | (d[pre + "type"] == 3)
            assert rel_linf(o["u"].reshape(3, -1), d[pre + "u"].reshape(3, -1), act) <= 1e-12, (name, step, "u")



@pytest.mark.parametrize("name", ["channel_bgk", "channel_movwall"])
def test_trt_with_equal_rates_matches_the_reference_bgk(name):
    """The TRT restatement (no reference counterpart) with the magic parameter
    (tau - 1/2)^2, so that both rates equal 1/tau, must reproduce the reference's BGK
    fixture to FP64 rounding."""
    from hybird_gb300 import abi
    d = load_golden(name)
    p = golden_params(d)
    tau = 0.5 + 3.0 * p.init_visc
    p.collision = abi.HB_TRT
    p.trt_magic = (tau - 0.5) ** 2
    sim = OracleSim(p)
    done = 0
    for step in d["steps"]:
        sim.cycle(int(step) - done)
        done = int(step)
        g = {k[len(f"s{step}_"):]: d[k] for k in d.files if k.startswith(f"s{step}_")}
        o = sim.lattice()
        act = (g["type"] == 0) | (g["type"] == 3)
        if "f" in g:
            assert rel_linf(o["f"].reshape(19, -1), g["f"].reshape(19, -1), act) <= 1e-13, (name, step)
        if step:
            assert rel_linf(o["u"].reshape(3, -1), g["u"].reshape(3, -1), act) <= 1e-12, (name, step)
