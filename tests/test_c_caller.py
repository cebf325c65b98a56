"""A compiled C++11 caller of the C-ABI (tests/c_caller/hb_caller.cpp): the header is
usable from the reference's language and standard (g++ -std=gnu++11, the reference's
own flags, nbproject/Makefile-Release.mk:52-53), the program links against the shared
library, and on a GPU its create -> init -> cycle -> download -> destroy sequence gives
the same state as the same run driven through the Python binding, and the FP64 oracle's
to rounding."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from hybird_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SRC = os.path.join(HERE, "c_caller", "hb_caller.cpp")


def _build(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    if not os.path.exists(abi.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    exe = tmp_path / "hb_caller"
    libdir = os.path.dirname(abi.LIB_PATH)
    subprocess.run(["g++", "-std=gnu++11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"),
                    SRC, "-o", str(exe), "-L", libdir, "-lhybird_gpu", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def test_c_caller_builds_against_the_header(tmp_path):
    assert _build(tmp_path).exists()


def _parse(out):
    vals = {}
    for line in out.strip().splitlines():
        tok = line.split()
        if tok[0] in ("x0", "x1", "FHydro", "MHydro"):
            vals[tok[0]] = np.array([float(t) for t in tok[1:]])
        else:
            for k in range(0, len(tok), 2):
                vals[tok[k]] = float(tok[k + 1])
    return vals


@pytest.mark.gpu
def test_c_caller_matches_python_binding_and_oracle(tmp_path):
    from hybird_gb300.gpu import GpuSim
    from oracle_port import OracleSim, rel_linf
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), str(abi.HB_FP64), "20"], check=True, capture_output=True, text=True).stdout
    got = _parse(out)
    p = abi.make_params((16, 16, 16), (7,) * 6, init_visc=0.1, lbF=(0.0, 0.0, -1e-4), multi_step=3,
                        collision=abi.HB_BGK, precision=abi.HB_FP64)
    spheres = np.array([[6.3, 7.1, 6.6, 2.5], [10.2, 9.4, 9.9, 2.2]])
    g = GpuSim(p, spheres)
    g.cycle(20)
    ge = g.elements()
    g.close()
    o = OracleSim(p, spheres)
    o.cycle(20)
    oe = o.elements()
    o.close()
    assert got["numeric"] == 0 and got["active"] == got["status_active"] and got["inside"] > 0
    for k in ("x0", "x1", "FHydro", "MHydro"):
        np.testing.assert_array_equal(got[k], ge[k], err_msg=k)  # the same library, the same run
        assert rel_linf(got[k], oe[k]) <= 1e-10, (k, rel_linf(got[k], oe[k]))
