"""CPU checks of the numpy discrete adjoint (oracle/vk_adjoint.py) that the GPU
adjoint is compared with: dot-product tests of the transposed pieces and
central finite differences (eps = 1e-6) of the gradient of final enstrophy
along seeded solenoidal directions."""

import numpy as np
import pytest

from oracle import vk_adjoint as va
from oracle import vk_oracle as vo
from vonkarman_gb300 import ics


def rdot(a, b):
    return float(sum((np.conj(x) * y).real.sum() for x, y in zip(a, b)))


def setup(n, seed=1):
    g = vo.Grid(n)
    ops = vo.SpectralOps(g)
    u0 = ops.leray_project(vo.hermitian_clean(g, vo.random_field(g, seed, amp=float(n) ** 3 / 8.0)))
    return g, ops, u0


def test_nonlinear_adjoint_dot_product():
    g, ops, x = setup(8)
    dx = vo.hermitian_clean(g, vo.random_field(g, 2, amp=10.0))
    y = vo.random_field(g, 3)
    e = 1e-6
    jp = vo.compute_nonlinear(ops, [a + e * b for a, b in zip(x, dx)])
    jm = vo.compute_nonlinear(ops, [a - e * b for a, b in zip(x, dx)])
    lhs = rdot(y, [(p - m) / (2 * e) for p, m in zip(jp, jm)])
    rhs = rdot(va.nonlinear_adjoint(ops, x, y), dx)
    assert abs(lhs - rhs) <= 1e-7 * abs(lhs)


def test_step_adjoint_dot_product():
    g, ops, u0 = setup(8)
    nu, dt = 0.05, 0.02
    s = vo.Periodic3D(g, nu, u0, dt_mode="fixed", dt_fixed=dt)
    v = ics.solenoidal_direction(8, seed=101)
    y = vo.random_field(g, 7)

    def stepmap(u):
        t = vo.Periodic3D(g, nu, u, dt_mode="fixed", dt_fixed=dt)
        t.step()
        return t.u_hat

    e = 1e-6
    jv = [(p - m) / (2 * e) for p, m in zip(stepmap([a + e * b for a, b in zip(u0, v)]),
                                               stepmap([a - e * b for a, b in zip(u0, v)]))]
    assert abs(rdot(y, jv) - rdot(va.step_adjoint(s, u0, y), v)) <= 1e-7 * abs(rdot(y, jv))


@pytest.mark.parametrize("n,nsteps", [(8, 5), (16, 3)])
def test_gradient_vs_central_fd(n, nsteps):
    g, ops, u0 = setup(n)
    nu, dt = 0.05, 0.02
    J, gw, _ = va.gradient(g, nu, dt, u0, nsteps)
    assert J > 0
    for seed in (1, 2, 3):
        v = ics.solenoidal_direction(n, seed=100 + seed)
        e = 1e-6
        jp, _ = va.forward_J(g, nu, dt, [a + e * b for a, b in zip(u0, v)], nsteps)
        jm, _ = va.forward_J(g, nu, dt, [a - e * b for a, b in zip(u0, v)], nsteps)
        fd = (jp - jm) / (2 * e)
        assert abs(fd - va.weighted_inner(g, v, gw)) <= 1e-6 * abs(fd)


def test_control_projection_is_idempotent_and_real():
    g, ops, u0 = setup(8)
    p = va.project_control(ops, vo.random_field(g, 4))
    q = va.project_control(ops, p)
    assert max(np.abs(a - b).max() for a, b in zip(p, q)) < 1e-12
    div = ops.KX * p[0] + ops.KY * p[1] + ops.KZ * p[2]
    assert np.abs(div).max() < 1e-12
    back = vo.hermitian_clean(g, p)
    assert max(np.abs(a - b).max() for a, b in zip(p, back)) < 1e-12
