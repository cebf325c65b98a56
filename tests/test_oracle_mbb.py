"""The moving bounce-back coupling in the oracle (not in the reference: its particle
branch is commented out, LB.cpp:1247-1276), pinned by a momentum-exchange identity.

A particle that does not move bounces populations back exactly as a fixed object does
(LB.cpp:535-550 makes objects static-wall nodes, BBi = 0), so its hydrodynamic force
must equal the object drag sum of 2 (fs_j - w_j) c_j over the fluid links into the
object (node::bounceBackForce, node.cpp:283-291): bit for bit while the particle is at
rest, and to rounding while a very heavy particle barely moves.  CPU only."""
import numpy as np

from hybird_gb300 import abi
from oracle_port import OracleSim


def _channel(coupling, dem_solve):
    # periodic x and z, walls at y; a decaying initial flow along x drives the fluid with
    # no body force, so the particle (DEM gravity is lbF, DEM.cpp:194) feels none
    return abi.make_params((28, 18, 16), (4, 4, 7, 7, 4, 4), init_visc=0.05, lbF=(0.0, 0.0, 0.0),
                           init_velocity=(0.02, 0.0, 0.004), multi_step=3, density=1e14,
                           dem_solve=dem_solve, coupling=coupling)


def test_moving_bounce_back_force_equals_object_drag():
    sphere = np.array([[13.3, 8.6, 7.7, 3.4]])
    obj = OracleSim(_channel(abi.HB_DIRECT_FORCING, 0), None, sphere)
    par = OracleSim(_channel(abi.HB_MOVING_BB, 1), sphere)
    lo, lp = obj.lattice(), par.lattice()
    # the same solid node set: object wall nodes and particle nodes
    np.testing.assert_array_equal(lo["type"] == 7, (lp["inside"] == 1) | (lp["type"] == 7))
    for step in range(1, 21):
        obj.cycle(1)
        par.cycle(1)
        drag = np.array([obj.object_drag(a) for a in range(3)])
        fh = par.elements()["FHydro"]
        assert np.abs(drag).max() > 0.0
        if step == 1:  # the particle has not moved yet
            np.testing.assert_array_equal(fh, drag)
        else:
            assert np.abs(fh - drag).max() <= 1e-12 * np.abs(drag).max(), (step, fh, drag)
    # the fluid away from the particle is the same flow
    lo, lp = obj.lattice(), par.lattice()
    fluid = (lo["type"] == 0) & (lp["inside"] == 0)
    assert np.abs(lo["u"].reshape(3, -1)[:, fluid] - lp["u"].reshape(3, -1)[:, fluid]).max() <= 1e-10


def test_moving_bounce_back_conserves_mass_of_a_still_particle():
    """No node is uncovered or covered while the particle is still, and bounce-back with
    BBi = 0 moves no mass: the fluid mass stays constant to rounding."""
    sphere = np.array([[13.3, 8.6, 7.7, 3.4]])
    par = OracleSim(_channel(abi.HB_MOVING_BB, 1), sphere)
    par.cycle(1)
    l0 = par.lattice()
    fl = (l0["type"] == 0) & (l0["inside"] == 0)
    m0 = l0["f"].reshape(19, -1)[:, fl].sum()
    par.cycle(30)
    l1 = par.lattice()
    np.testing.assert_array_equal(l1["inside"], l0["inside"])
    m1 = l1["f"].reshape(19, -1)[:, fl].sum()
    assert abs(m1 - m0) <= 1e-11 * m0
