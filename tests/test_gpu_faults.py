"""Failures made on the host, reported by the library as status codes (the reference
exits instead: macros.h:8, LB.cpp:1057, 1460).  None of these faults, traps or hangs the
GPU: each bad input is one the device code bounds-checks or computes through.

  * a candidate list smaller than a particle's neighbours (hb_params.cap_neighbors);
  * an interface list smaller than the free surface (hb_params.cap_interface);
  * a NaN population in an uploaded lattice state;
  * a particle outside the box (outside the DEM cell grid, DEM.cpp:1326-1367)."""
import numpy as np
import pytest

from hybird_gb300 import abi
from oracle_port import golden_gasbox, golden_params, load_golden

pytestmark = pytest.mark.gpu


def _gpu():
    from hybird_gb300.gpu import GpuSim, HbError
    return GpuSim, HbError


def _cluster():
    """Six small spheres within nebrRange of each other in a closed 16^3 box."""
    c = np.array([[6.0, 6.0, 6.0], [9.5, 6.0, 6.0], [6.0, 9.5, 6.0], [9.5, 9.5, 6.0], [6.0, 6.0, 9.5], [9.5, 9.5, 9.5]])
    return np.c_[c, np.full(len(c), 1.5)]


def test_candidate_list_capacity_is_reported():
    GpuSim, HbError = _gpu()
    p = abi.make_params((16, 16, 16), (7,) * 6, lbF=(0, 0, -1e-4), multi_step=3, cap_neighbors=2)
    g = GpuSim(p, _cluster())
    with pytest.raises(HbError, match="candidate list full"):
        g.cycle(1)
    st = g.status()
    assert st.capacity_error & 1
    g.close()
    # the default capacity holds the same particles
    g = GpuSim(abi.make_params((16, 16, 16), (7,) * 6, lbF=(0, 0, -1e-4), multi_step=3), _cluster())
    g.cycle(2)
    assert g.status().capacity_error == 0 and g.status().pairs == 6  # the oracle finds 6
    g.close()


def test_interface_list_capacity_is_reported():
    GpuSim, HbError = _gpu()
    d = load_golden("dambreak_fs")
    p = golden_params(d, gas_box=golden_gasbox("dambreak_fs"), cap_interface=8)
    g = GpuSim(p)
    with pytest.raises(HbError, match="interface list full"):
        g.cycle(1)
    assert g.status().capacity_error & 8
    g.close()


def test_nan_in_uploaded_populations_is_reported():
    GpuSim, HbError = _gpu()
    p = abi.make_params((12, 10, 8), (4, 4, 7, 7, 4, 4), lbF=(1e-6, 0, 0), dem_solve=0)
    g = GpuSim(p)
    g.cycle(2)
    st = g.lattice()
    f = st["f"].copy()
    node = 5 + 12 * (4 + 10 * 3)  # an interior fluid node
    assert st["type"][node] == 0
    f[7 * g.N + node] = np.nan
    g.upload(st["type"], st["inside"], st["solid"], f, st["n"], st["u"], st["mass"])
    with pytest.raises(HbError, match="NaN"):
        g.cycle(1)
    assert g.status().numeric_error != 0
    g.close()


def test_particle_outside_the_box_is_reported():
    GpuSim, HbError = _gpu()
    p = abi.make_params((16, 16, 16), (7,) * 6, lbF=(0, 0, -1e-4), multi_step=3, lb_solve=0)
    spheres = np.array([[8.0, 8.0, 8.0, 2.0], [8.0, 8.0, -30.0, 2.0]])
    g = GpuSim(p, spheres)
    with pytest.raises(HbError, match="outside the DEM cell grid"):
        g.cycle(1)
    assert g.status().capacity_error & 2
    g.close()
