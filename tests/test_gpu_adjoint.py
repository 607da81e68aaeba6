"""GPU discrete adjoint against the numpy adjoint (oracle/vk_adjoint.py) and
central finite differences of the GPU forward map.  Tolerances: 1e-11
norm-relative for the transposed nonlinear term and the gradient vs the numpy
adjoint (FP64), 1e-6 relative for central FD (eps = 1e-6), 1e-4 for the
FP32-bulk gradient against the FP64 one."""

import math

import numpy as np
import pytest

from oracle import vk_adjoint as va
from oracle import vk_oracle as vo

pytestmark = pytest.mark.gpu


def nrel(a, b):
    num = math.sqrt(sum(float(np.sum(np.abs(x - y) ** 2)) for x, y in zip(a, b)))
    den = math.sqrt(sum(float(np.sum(np.abs(y) ** 2)) for y in b))
    return num / den


@pytest.fixture(scope="module")
def vk():
    import vonkarman_gb300 as vk

    return vk


def state(n, seed=1):
    g = vo.Grid(n)
    ops = vo.SpectralOps(g)
    return g, ops, ops.leray_project(vo.hermitian_clean(g, vo.random_field(g, seed, amp=float(n) ** 3 / 40.0)))


@pytest.mark.parametrize("n", [8, 16, 32])
def test_nonlinear_adjoint_vs_oracle(vk, n):
    g, ops, x = state(n)
    nbar = vo.random_field(g, 5)
    want = va.nonlinear_adjoint(ops, x, nbar)
    s = vk.Periodic3D(vk.GridSpec(n), 0.05, x, vk.SolverOptions(dt_mode="fixed", dt_fixed=0.02))
    assert nrel(vk.nonlinear_adjoint(s, x, nbar), want) < 1e-11


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32bulk", 2e-5)])
def test_nonlinear_adjoint_vs_oracle_n128(vk, precision, tol):
    n = 128
    g, ops, x = state(n)
    nbar = vo.random_field(g, 6)
    want = va.nonlinear_adjoint(ops, x, nbar)
    s = vk.Periodic3D(vk.GridSpec(n), 0.05, x, vk.SolverOptions(precision=precision, dt_mode="fixed",
                                                                  dt_fixed=0.02))
    assert nrel(vk.nonlinear_adjoint(s, x, nbar), want) < tol
    s.close()


@pytest.mark.parametrize("n,nsteps,nsnap", [(8, 5, 5), (16, 3, 2), (16, 6, 1)])
def test_gradient_vs_oracle(vk, n, nsteps, nsnap):
    g, ops, u0 = state(n)
    nu, dt = 0.05, 0.02
    J, gw, _ = va.gradient(g, nu, dt, u0, nsteps)
    s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=dt))
    Jg = s.adjoint_forward(nsteps, nsnap)
    assert abs(Jg - J) <= 1e-11 * J
    assert nrel(s.adjoint_backward(), gw) < 1e-10


def test_checkpoint_schedule_does_not_change_gradient(vk):
    n, nu, dt, nsteps = 16, 0.05, 0.02, 7
    g, ops, u0 = state(n, 3)
    grads = []
    for nsnap in (1, 3, 7):
        s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=dt))
        s.adjoint_forward(nsteps, nsnap)
        grads.append(s.adjoint_backward())
    for gr in grads[1:]:
        for a, b in zip(gr, grads[0]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("nsnap", [1, 2, 3, 7])
def test_binomial_schedule_gives_the_two_level_gradient(vk, nsnap):
    # treeverse over nsnap slots (vk_adjoint_set_schedule) against the
    # two-level schedule: the same steps in the same order, bitwise
    n, nu, dt, nsteps = 16, 0.05, 0.02, 7
    g, ops, u0 = state(n, 3)
    out = {}
    for sch in ("two-level", "binomial"):
        s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=dt))
        J = s.adjoint_forward(nsteps, nsnap, schedule=sch)
        out[sch] = (J, s.adjoint_backward())
        s.close()
    assert out["binomial"][0] == out["two-level"][0]
    for a, b in zip(out["binomial"][1], out["two-level"][1]):
        assert np.array_equal(a, b)


def test_gradient_vs_central_fd_on_gpu(vk):
    from vonkarman_gb300 import ics

    n, nu, dt, nsteps = 32, 0.02, 5e-3, 12
    g, ops, u0 = state(n, 4)
    opts = vk.SolverOptions(dt_mode="fixed", dt_fixed=dt)
    s = vk.Periodic3D(vk.GridSpec(n), nu, u0, opts)
    s.adjoint_forward(nsteps, 3)
    grad = s.adjoint_backward()

    def J(u):
        t = vk.Periodic3D(vk.GridSpec(n), nu, u, opts)
        return t.adjoint_forward(nsteps, 1)

    for seed in (1, 2, 3):
        v = ics.solenoidal_direction(n, seed=200 + seed)
        e = 1e-6
        fd = (J([a + e * b for a, b in zip(u0, v)]) - J([a - e * b for a, b in zip(u0, v)])) / (2 * e)
        assert abs(fd - vk.l2_inner(v, grad, n)) <= 1e-6 * abs(fd)


def test_fp32bulk_gradient_vs_fp64(vk):
    n, nu, dt, nsteps = 32, 0.02, 5e-3, 10
    g, ops, u0 = state(n, 6)
    grads = []
    for prec in ("fp64", "fp32bulk"):
        s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(precision=prec, dt_mode="fixed", dt_fixed=dt))
        s.adjoint_forward(nsteps, 2)
        grads.append(s.adjoint_backward())
    assert nrel(grads[1], grads[0]) < 1e-4


@pytest.mark.parametrize("n", [256, 512])
def test_fp32bulk_gradient_vs_fp64_large_grids(vk, n):
    # the 384- and 768-point plans of the adjoint chain (A1..A5), both forms
    # against each other (the oracle is too slow at these sizes)
    from vonkarman_gb300 import ics

    nu, dt, nsteps = 2e-3, 1e-3, 2
    u0 = ics.project_control(ics.von_karman_isotropic(n, kp=3.0, energy=0.5, seed=7), n)
    out = []
    for prec in ("fp64", "fp32bulk"):
        s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(precision=prec, dt_mode="fixed", dt_fixed=dt))
        J = s.adjoint_forward(nsteps, 1)
        out.append((J, s.adjoint_backward()))
        s.close()
    (j64, g64), (j32, g32) = out
    assert abs(j32 - j64) <= 1e-5 * abs(j64)
    assert nrel(g32, g64) < 1e-4


def test_adjoint_rejects_cfl_mode(vk):
    from vonkarman_gb300._native import VkError

    n = 8
    g, ops, u0 = state(n)
    s = vk.Periodic3D(vk.GridSpec(n), 0.05, u0)
    with pytest.raises(VkError):
        s.adjoint_forward(2, 1)
