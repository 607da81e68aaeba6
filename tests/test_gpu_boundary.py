"""GPU checks of the boundary entry points beyond the stepper: the
SpectralOps fields and apply_viscous against the oracle (bit-identical in
FP64: same formulas, each operation rounded once), and the non-finite state
report.  The non-finite case is injected on the host: a state with one NaN
coefficient is uploaded through the C ABI; no kernel faults."""

import math

import numpy as np
import pytest

from oracle import vk_oracle as vo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,l", [(16, 2.0 * math.pi), (32, 3.0), (64, 2.0 * math.pi)])
def test_spectral_ops_fields_bitwise(n, l):
    import vonkarman_gb300 as vk

    g = vo.Grid(n, l)
    ops = vo.SpectralOps(g)
    u0 = vo.taylor_green(g)
    s = vk.Periodic3D(vk.GridSpec(n, l), 0.01, u0)
    got = vk.spectral_ops(s)
    assert np.array_equal(got.kx, ops.kx)
    assert np.array_equal(got.ky, ops.ky)
    assert np.array_equal(got.kz, ops.kz)
    assert np.array_equal(got.k_mag_sq, ops.k_mag_sq)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32bulk"])
def test_apply_viscous_vs_oracle(precision):
    import vonkarman_gb300 as vk

    n, nu = 32, 0.013
    g = vo.Grid(n, 2.5)
    ops = vo.SpectralOps(g)
    u = vo.hermitian_clean(g, vo.random_field(g, 21, amp=3.0))
    s = vk.Periodic3D(vk.GridSpec(n, 2.5), 0.01, u, vk.SolverOptions(precision=precision))
    got = vk.apply_viscous(s, u, nu)
    want = ops.apply_viscous(u, nu)
    if precision == "fp64":
        for a, b in zip(got, want):
            assert np.array_equal(a, b)
    else:
        num = max(float(np.abs(a - b).max()) for a, b in zip(got, want))
        assert num <= 1e-6 * max(float(np.abs(b).max()) for b in want)
    if precision == "fp64":   # the solver state is untouched
        assert all(np.array_equal(a, b) for a, b in zip(s.u_hat(), u))
    s.close()


@pytest.mark.parametrize("dt_mode", ["cfl", "fixed"])
def test_nonfinite_state_is_reported(dt_mode):
    import vonkarman_gb300 as vk
    from vonkarman_gb300._native import VkError

    n = 16
    g = vo.Grid(n)
    u0 = vo.taylor_green(g)
    bad = [c.copy() for c in u0]
    bad[1][3, 2, 1] = complex(float("nan"), 0.0)
    opts = vk.SolverOptions(dt_mode=dt_mode, dt_fixed=1e-3)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, opts)
    s.step(2)
    assert math.isfinite(s.time())
    s.restore_state(bad, 0.0, 0, 1e-3)
    s.step(1)
    with pytest.raises(VkError) as ei:
        s.time()
    assert ei.value.code == 6  # VK_ERR_NONFINITE
    with pytest.raises(VkError):
        s.run(2, every=1)
    # a finite state clears the condition
    s.restore_state(u0, 0.0, 0, 1e-3)
    s.step(1)
    assert s.time() > 0.0
    s.close()
