"""Reverse (adjoint) entry points: the object drag J and its gradient with respect to the
body force, the relaxation time and the inlet field.

Pins: (1) the forward J against the CPU oracle's drag (FP64 reference-order lattice step
plus node::bounceBackForce summed over object links); (2) the FP64 gradient against
central finite differences of the FP64 forward (relative step 1e-4); (3) checkpoint
spacing changes nothing (bit-identical); (4) the FP32 gradient against the FP64 one and
against finite differences (1e-4 relative is the stated target)."""
import numpy as np
import pytest

from hybird_gb300 import abi
from hybird_gb300.workloads import adjoint_channel
from oracle_port import OracleSim

pytestmark = pytest.mark.gpu

SMALL = dict(shape=(34, 22, 20), per_axis=2, radius=4.0, jitter=1.5, seed=3, tau=0.7, force=1e-5,
             u0=0.03, zwave=0.2)


def _gpu(params, objects):
    from hybird_gb300.gpu import GpuSim
    return GpuSim(params, None, objects)


def _central(f, h):
    return (f(h) - f(-h)) / (2.0 * h)


def test_forward_drag_matches_oracle():
    p, obj, uin = adjoint_channel(precision=abi.HB_FP64, **SMALL)
    T = 40
    g = _gpu(p, obj)
    J = g.adjoint_forward(T, tau=0.7, force=tuple(p.lbF), inlet=uin, precision=abi.HB_FP64)
    o = OracleSim(p, None, obj)
    o.set_inlet(uin)
    o.cycle(T)
    Jo = o.object_drag(0)
    assert abs(Jo) > 0.0
    assert abs(J - Jo) <= 1e-11 * abs(Jo), (J, Jo)
    g.close()


def test_fp64_gradient_matches_finite_differences():
    p, obj, uin = adjoint_channel(precision=abi.HB_FP64, **SMALL)
    T, K, tau = 60, 16, 0.7
    F = np.array(p.lbF[:])
    g = _gpu(p, obj)
    J, dF, dtau, duin = g.adjoint_drag(T, tau, F, uin, abi.HB_FP64, K)
    fwd = lambda tau_, F_, u_: g.adjoint_forward(T, tau_, F_, u_, abi.HB_FP64, K)
    assert abs(J - fwd(tau, F, uin)) <= 1e-14 * abs(J)
    h = 1e-4
    fd_tau = _central(lambda e: fwd(tau + e, F, uin), h * tau)
    fd_Fx = _central(lambda e: fwd(tau, F + np.array([e, 0, 0]), uin), h * F[0])
    fd_Fy = _central(lambda e: fwd(tau, F + np.array([0, e, 0]), uin), h * F[0])
    rng = np.random.default_rng(11)
    v = rng.uniform(-1.0, 1.0, size=uin.shape)
    fd_v = _central(lambda e: fwd(tau, F, uin + e * v), h * np.abs(uin).max())
    assert abs(dtau - fd_tau) <= 1e-6 * abs(fd_tau), (dtau, fd_tau)
    assert abs(dF[0] - fd_Fx) <= 1e-6 * abs(fd_Fx), (dF[0], fd_Fx)
    assert abs(dF[1] - fd_Fy) <= 1e-6 * abs(fd_Fx), (dF[1], fd_Fy)
    assert abs(duin @ v - fd_v) <= 1e-6 * abs(fd_v), (duin @ v, fd_v)
    # single inlet entries, on the largest-gradient node and on one near a wall
    X, Y, Z = p.lb_size
    for q in (int(np.argmax(np.abs(duin))), 2 + Y * 5):
        e_q = np.zeros_like(uin)
        e_q[q] = 1.0
        fd_q = _central(lambda e: fwd(tau, F, uin + e * e_q), h * np.abs(uin).max())
        assert abs(duin[q] - fd_q) <= 1e-6 * np.abs(duin).max(), (q, duin[q], fd_q)
    g.close()


def test_checkpoint_spacing_does_not_change_the_gradient():
    p, obj, uin = adjoint_channel(precision=abi.HB_FP32, **SMALL)
    g = _gpu(p, obj)
    F = tuple(p.lbF)
    res = [g.adjoint_drag(37, 0.7, F, uin, abi.HB_FP32, K) for K in (37, 5, 1)]
    for r in res[1:]:
        assert r[0] == res[0][0]
        np.testing.assert_array_equal(r[1], res[0][1])
        assert r[2] == res[0][2]
        np.testing.assert_array_equal(r[3], res[0][3])
    g.close()


def test_fp32_gradient_against_fp64_adjoint():
    p, obj, uin = adjoint_channel(precision=abi.HB_FP32, **SMALL)
    g = _gpu(p, obj)
    F = tuple(p.lbF)
    J32, dF32, dt32, du32 = g.adjoint_drag(60, 0.7, F, uin, abi.HB_FP32, 16)
    J64, dF64, dt64, du64 = g.adjoint_drag(60, 0.7, F, uin, abi.HB_FP64, 16)
    assert abs(J32 - J64) <= 1e-4 * abs(J64)
    assert abs(dt32 - dt64) <= 1e-4 * abs(dt64), (dt32, dt64)
    assert abs(dF32[0] - dF64[0]) <= 1e-4 * abs(dF64[0]), (dF32, dF64)
    assert np.linalg.norm(du32 - du64) <= 1e-4 * np.linalg.norm(du64)
    g.close()


def test_adjoint_rejects_unsupported_lattices():
    from hybird_gb300.gpu import GpuSim, HbError
    spheres = np.array([[10.0, 10.0, 10.0, 3.0]])
    p = abi.make_params((20, 20, 20), (7,) * 6, init_visc=0.1)
    g = GpuSim(p, spheres)
    with pytest.raises(HbError, match="UNSUPPORTED|unsupported|particles"):
        g.adjoint_drag(5, 0.8, (0, 0, 0))
    g.close()
