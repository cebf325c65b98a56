"""The moving bounce-back coupling (hb_params.coupling = HB_MOVING_BB) on the GPU against
the FP64 oracle's restatement of it (oracle/hb_oracle.cpp; the oracle itself is pinned by
the momentum-exchange identity in tests/test_oracle_mbb.py, since the reference has no
such mode: its particle branch is commented out, LB.cpp:1247-1276).

Spheres settle in a closed box, so nodes are uncovered (refilled) and covered every few
steps.  Exact: node types, particle flags, particle indices and the solid-node counts
(fluidVolume).  FP64 populations and velocity to 1e-12 relative L-inf over the fluid
nodes, element force and torque to 1e-10 (the force is summed per particle in a fixed
tree instead of in node order).  FP32 and FP16-storage velocity error against the FP64
oracle as for the direct-forcing form."""
import numpy as np
import pytest

from hybird_gb300 import abi
from oracle_port import OracleSim, rel_linf

pytestmark = pytest.mark.gpu


def _gpu():
    from hybird_gb300.gpu import GpuSim
    return GpuSim


def _box(precision=abi.HB_FP64, collision=abi.HB_BGK):
    rng = np.random.default_rng(11)
    spheres = []
    while len(spheres) < 10:
        r = rng.uniform(2.5, 3.5)
        c = rng.uniform(2 + r, 30 - r, size=3)
        if all(np.linalg.norm(c - s[:3]) > r + s[3] + 0.5 for s in spheres):
            spheres.append(np.r_[c, r])
    p = abi.make_params((32, 32, 32), (7,) * 6, init_visc=0.1, lbF=(0, 0, -3e-4), multi_step=3,
                        collision=collision, precision=precision, coupling=abi.HB_MOVING_BB)
    return p, np.array(spheres)


def _solid_fluid(l):
    fluid = ((l["type"] == 0) | (l["type"] == 3)) & (l["inside"] == 0)
    return fluid


@pytest.mark.parametrize("collision", [abi.HB_BGK, abi.HB_TRT])
def test_moving_bounce_back_fp64_vs_oracle(collision):
    p, spheres = _box(collision=collision)
    g = _gpu()(p, spheres)
    o = OracleSim(p, spheres, threads=4)
    changed = 0
    prev = None
    for step in (1, 10, 30, 60):
        done = 0 if prev is None else prev[0]
        g.cycle(step - done)
        o.cycle(step - done)
        gl, ol = g.lattice(), o.lattice()
        np.testing.assert_array_equal(gl["type"], ol["type"])
        np.testing.assert_array_equal(gl["inside"], ol["inside"], err_msg=f"step {step}")
        ins = ol["inside"] == 1
        np.testing.assert_array_equal(gl["solid"][ins], ol["solid"][ins])
        if prev is not None:
            changed += int((prev[1] != ol["inside"]).sum())
        prev = (step, ol["inside"].copy())
        fl = _solid_fluid(ol)
        ef = rel_linf(gl["f"].reshape(19, -1), ol["f"].reshape(19, -1), fl)
        eu = rel_linf(gl["u"].reshape(3, -1), ol["u"].reshape(3, -1), fl)
        ge, oe = g.elements(), o.elements()
        efh = rel_linf(ge["FHydro"], oe["FHydro"])
        emh = rel_linf(ge["MHydro"], oe["MHydro"])
        print(f"mbb step {step}: f {ef:.2e} u {eu:.2e} FHydro {efh:.2e} MHydro {emh:.2e}")
        assert ef <= 1e-12 and eu <= 1e-12, (step, ef, eu)
        assert efh <= 1e-10 and emh <= 1e-10, (step, efh, emh)
        np.testing.assert_array_equal(ge["fluidVolume"], oe["fluidVolume"])
        assert rel_linf(ge["x0"], oe["x0"]) <= 1e-12
    assert changed > 0  # particles uncovered and covered nodes over the run
    g.close()
    o.close()


@pytest.mark.parametrize("prec,tol", [(abi.HB_FP32, 1e-5), (abi.HB_FP16S, 5e-2)])
def test_moving_bounce_back_reduced_precision_vs_fp64_oracle(prec, tol):
    p64, spheres = _box()
    p, _ = _box(precision=prec)
    g = _gpu()(p, spheres)
    o = OracleSim(p64, spheres, threads=4)
    g.cycle(100)
    o.cycle(100)
    gl, ol = g.lattice(), o.lattice()
    np.testing.assert_array_equal(gl["inside"], ol["inside"])
    fl = _solid_fluid(ol)
    du = gl["u"].reshape(3, -1)[:, fl] - ol["u"].reshape(3, -1)[:, fl]
    l2 = np.sqrt((du ** 2).sum() / (ol["u"].reshape(3, -1)[:, fl] ** 2).sum())
    ge, oe = g.elements(), o.elements()
    print(f"mbb prec {prec}: u rel L2 {l2:.3e}, FHydro {rel_linf(ge['FHydro'], oe['FHydro']):.3e}")
    assert l2 <= tol, l2
    assert rel_linf(ge["x0"], oe["x0"]) <= 1e-4
    g.close()
    o.close()


def test_moving_bounce_back_rejects_periodic_faces():
    from hybird_gb300.gpu import HbError
    p = abi.make_params((24, 16, 16), (4, 4, 7, 7, 7, 7), lbF=(1e-5, 0, 0), multi_step=3,
                        coupling=abi.HB_MOVING_BB)
    with pytest.raises(HbError, match="moving bounce-back"):
        _gpu()(p, np.array([[12.0, 8.0, 8.0, 3.0]]))
