"""Pins the numpy oracle against the reference's own known-answer and invariant
tests for the hot path.  Each test names the reference test it restates
(file:line in alejandro-soto-franco/vonkarman).  CPU only."""

import math

import numpy as np
import pytest

from oracle import vk_oracle as vo

TWO_PI = 2.0 * math.pi


# vonkarman-core/src/spectral_ops.rs:183-195  wavenumbers_n8
def test_wavenumbers_n8():
    ops = vo.SpectralOps(vo.Grid(8))
    assert len(ops.kx) == 8
    assert abs(ops.kx[0]) < 1e-14
    assert abs(ops.kx[1] - 1.0) < 1e-14
    assert abs(ops.kx[4] + 4.0) < 1e-14
    assert abs(ops.kx[7] + 1.0) < 1e-14
    assert len(ops.kz) == 5
    assert abs(ops.kz[4] - 4.0) < 1e-14


# spectral_ops.rs:197-202  k_mag_sq_shape
def test_k_mag_sq_shape():
    ops = vo.SpectralOps(vo.Grid(8))
    assert ops.k_mag_sq.shape == (8, 8, 5)


# spectral_ops.rs:204-235  leray_divergence_free
def test_leray_divergence_free():
    g = vo.Grid(8)
    ops = vo.SpectralOps(g)
    shp = g.spectral_shape
    u = [np.full(shp, 1 + 1j), np.full(shp, 2 + 1j), np.full(shp, 3 + 1j)]
    u = ops.leray_project(u)
    div = ops.KX * u[0] + ops.KY * u[1] + ops.KZ * u[2]
    assert np.abs(div).max() < 1e-12


# spectral_ops.rs:237-260  curl_of_constant_is_zero
def test_curl_of_constant_is_zero():
    g = vo.Grid(8)
    ops = vo.SpectralOps(g)
    u = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    u[0][0, 0, 0] = 5.0
    for c in ops.curl(u):
        assert np.abs(c).max() < 1e-14


# vonkarman-fft/src/ndrustfft_backend.rs:75-106  roundtrip_identity
def test_fft_roundtrip_identity():
    n = 8
    x = np.sin(TWO_PI * np.arange(n) / n)[:, None, None] * np.ones((n, n, n))
    back = vo.c2r_3d(vo.r2c_3d(x), (n, n, n))
    assert np.abs(back - x).max() < 1e-12


# ndrustfft_backend.rs:108-147  parseval_theorem
def test_fft_parseval():
    n = 16
    i = np.arange(n)
    x = (np.sin(TWO_PI * i / n)[:, None, None] + np.cos(TWO_PI * i / n)[None, :, None]) * np.ones((n, n, n))
    phys = float((x * x).sum())
    s = vo.r2c_3d(x)
    w = np.full(n // 2 + 1, 2.0)
    w[0] = w[-1] = 1.0
    spec = float((w * (s.real ** 2 + s.imag ** 2)).sum()) / n ** 3
    assert abs(phys - spec) / phys < 1e-10


# vonkarman-fft/src/dealiased.rs:173-202  dealiased_cross_product_zero_input
def test_dealiased_zero_input():
    g = vo.Grid(8)
    z = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    for c in vo.dealiased_cross_product(g, z, z):
        assert np.abs(c.real).max() < 1e-14 and np.abs(c.imag).max() < 1e-14


# dealiased.rs:204-263  cross_product_anti_symmetry
def test_cross_product_antisymmetry():
    g = vo.Grid(8)
    u = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    o = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    u[0][1, 0, 0] = 1.0 + 0.5j
    o[1][0, 1, 0] = 0.7 - 0.3j
    r1 = vo.dealiased_cross_product(g, u, o)
    r2 = vo.dealiased_cross_product(g, o, u)
    for a, b in zip(r1, r2):
        assert np.abs((a + b).real).max() < 1e-10 and np.abs((a + b).imag).max() < 1e-10


# vonkarman-periodic/src/nonlinear.rs:50-97  nonlinear_term_divergence_free
def test_nonlinear_divergence_free():
    g = vo.Grid(16)
    ops = vo.SpectralOps(g)
    u = vo.taylor_green(g)
    nl = vo.compute_nonlinear(ops, u)
    div = ops.KX * nl[0] + ops.KY * nl[1] + ops.KZ * nl[2]
    assert np.abs(div).max() < 1e-6


# vonkarman-periodic/src/etd.rs:142-213
def test_phi_known_values():
    assert abs(vo.phi1(0.0) - 1.0) < 1e-12  # etd.rs:142-146
    assert abs(vo.phi2(0.0) - 0.5) < 1e-12  # etd.rs:148-152
    assert abs(vo.phi1(1.0) - (math.e - 1.0)) < 1e-10  # etd.rs:154-162
    assert abs(vo.phi2(1.0) - (math.e - 2.0)) < 1e-10  # etd.rs:164-172
    exp100 = (math.exp(-100.0) - 1.0) / -100.0
    assert abs(vo.phi1(-100.0) - exp100) / abs(exp100) < 1e-8  # etd.rs:174-182
    for z in (1e-10, 1e-8, 1e-6, 1e-4, 1e-2):  # etd.rs:184-198
        assert abs(vo.phi1(z) - 1.0) < abs(z) * 2.0
        assert abs(vo.phi2(z) - 0.5) < abs(z) * 2.0
    c = vo.EtdCoeffs.new(0.0)  # etd.rs:200-213
    assert abs(c.exp_full - 1.0) < 1e-12 and abs(c.exp_half - 1.0) < 1e-12
    assert abs(c.b1 + 2.0 * c.b23 + c.b4 - 1.0) < 1e-10


# vonkarman-periodic/src/solver.rs:625-650  taylor_green_energy_decays
def test_taylor_green_energy_decays():
    g = vo.Grid(16)
    s = vo.Periodic3D(g, 0.01, vo.taylor_green(g))
    e0 = s.energy()
    assert e0 > 0
    prev = e0
    for _ in range(50):
        s.step()
        e = s.energy()
        assert e <= prev + 1e-14 * max(abs(prev), 1e-30)
        prev = e
    assert prev < 0.99 * e0


# solver.rs:652-671  taylor_green_short_time_exponential_decay
def test_taylor_green_short_time_decay():
    g = vo.Grid(32)
    nu = 0.01
    s = vo.Periodic3D(g, nu, vo.taylor_green(g))
    e0 = s.energy()
    while s.time < 0.5:
        s.step()
    expected = e0 * math.exp(-2.0 * nu * s.time)
    assert abs(s.energy() - expected) / expected < 0.1


# solver.rs:673-706 and tests/checkpoint_restart.rs:10-63  bitwise restart
def test_checkpoint_restart_bitwise():
    g = vo.Grid(16)
    u0 = vo.taylor_green(g)
    cont = vo.Periodic3D(g, 0.01, u0)
    for _ in range(20):
        cont.step()
    half = vo.Periodic3D(g, 0.01, u0)
    for _ in range(10):
        half.step()
    rest = vo.Periodic3D(g, 0.01, half.u_hat, time=half.time, step_count=half.step_count, dt=half.dt)
    for _ in range(10):
        rest.step()
    for a, b in zip(cont.u_hat, rest.u_hat):
        assert np.array_equal(a, b)
    assert cont.time == rest.time and cont.step_count == rest.step_count


# vonkarman-periodic/src/rk4.rs:155-214  rk4_energy_decays
def test_rk4_energy_decays():
    g = vo.Grid(16)
    ops = vo.SpectralOps(g)
    u = vo.taylor_green(g)
    e0 = vo.spectral_energy(g, u)
    prev = e0
    for _ in range(20):
        u = vo.rk4_step(u, ops, 0.01, 0.001)
        e = vo.spectral_energy(g, u)
        assert e <= prev + 1e-12 * max(abs(prev), 1e-30)
        prev = e
    assert prev < 0.999 * e0


# vonkarman-diag/src/spectrum.rs:92-136  spectrum_single_mode
def test_spectrum_single_mode():
    n = 8
    g = vo.Grid(n)
    ops = vo.SpectralOps(g)
    u = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    u[0][1, 0, 0] = -0.5j * n ** 3
    u[0][n - 1, 0, 0] = 0.5j * n ** 3
    shells, spec = vo.energy_spectrum(u, ops)
    assert spec[1] > 0
    assert abs(spec[0]) < 1e-10
    assert np.all(np.abs(spec[2:]) < 1e-10)
    assert len(shells) == vo.n_shells(g) == 8  # ceil(sqrt(3)*4)+1


# spectrum.rs:138-200  spectrum_total_equals_energy
def test_spectrum_total_equals_energy():
    g = vo.Grid(16)
    ops = vo.SpectralOps(g)
    u = vo.taylor_green(g)
    _, spec = vo.energy_spectrum(u, ops)
    direct = vo.spectral_energy(g, u)
    assert abs(spec.sum() - direct) / direct < 1e-10


# ic/taylor_green.rs:54-78 (E=1/8) and ic/abc.rs:66-96 (E=1.5)
def test_ic_energies():
    assert abs(vo.spectral_energy(vo.Grid(32), vo.taylor_green(vo.Grid(32))) - 0.125) < 1e-6
    assert abs(vo.spectral_energy(vo.Grid(32), vo.abc_flow(vo.Grid(32))) - 1.5) < 1e-6


# tests/convergence.rs:34-78  spectral_convergence_taylor_green
def test_convergence_taylor_green():
    nu, t_final = 0.1, 0.1
    errs = []
    for n in (8, 16, 32, 64):
        g = vo.Grid(n)
        s = vo.Periodic3D(g, nu, vo.taylor_green(g))
        while s.time < t_final:
            s.step()
        expected = 0.125 * math.exp(-6.0 * nu * s.time)
        err = abs(s.energy() - expected) / expected
        assert err < 0.05
        errs.append(err)
    assert max(errs) < 10.0 * min(errs)


# tests/convergence.rs:80-127  parseval_identity_all_grid_sizes
def test_parseval_all_sizes():
    for n in (8, 16, 32):
        g = vo.Grid(n)
        u = vo.taylor_green(g)
        e_spec = vo.spectral_energy(g, u)
        e_phys = 0.5 * sum(float((vo.c2r_3d(c, (n,) * 3) ** 2).sum()) for c in u) / n ** 3
        assert abs(e_spec - e_phys) / e_spec < 1e-12


# tests/energy_budget.rs:12-66  energy_budget_taylor_green
def test_energy_budget_taylor_green():
    g = vo.Grid(32)
    nu = 0.01
    s = vo.Periodic3D(g, nu, vo.taylor_green(g))
    for _ in range(10):
        s.step()
    prev_e, prev_ens, ok = s.energy(), s.enstrophy(), 0
    for _ in range(50):
        dt = s.dt
        s.step()
        e, ens = s.energy(), s.enstrophy()
        expected = -2.0 * nu * 0.5 * (prev_ens + ens)
        res = abs((e - prev_e) / dt - expected) / max(abs(expected), 1e-30)
        ok += res < 0.6
        prev_e, prev_ens = e, ens
    assert ok / 50.0 > 0.9


# tests/energy_budget.rs:68-106  helicity_conservation_abc_flow
def test_helicity_abc_flow_decays():
    g = vo.Grid(32)
    s = vo.Periodic3D(g, 0.01, vo.abc_flow(g))
    h0 = s.helicity()
    assert abs(h0) > 0.1
    for _ in range(30):
        s.step()
    assert abs(s.helicity()) < abs(h0)
    assert s.energy() < 1.5


# tests/taylor_green_re100.rs:6-52 (monotone decay, |H| < 1e-10) and :54-80
def test_taylor_green_re100():
    g = vo.Grid(16)
    nu = 0.01
    s = vo.Periodic3D(g, nu, vo.taylor_green(g))
    e0 = prev = s.energy()
    for _ in range(100):
        s.step()
        e = s.energy()
        assert np.isfinite(e) and e <= prev + 1e-12 * max(abs(prev), 1e-30)
        prev = e
    assert prev < 0.9 * e0
    assert s.enstrophy() > 0
    assert abs(s.helicity()) < 1e-10


def test_taylor_green_dissipation_consistency():
    # tests/taylor_green_re100.rs:54-80
    g = vo.Grid(16)
    nu = 0.01
    s = vo.Periodic3D(g, nu, vo.taylor_green(g))
    for _ in range(20):
        s.step()
    e1, ens, dt = s.energy(), s.enstrophy(), s.dt
    s.step()
    rate = (s.energy() - e1) / dt
    assert abs(rate - (-2.0 * nu * ens)) / abs(2.0 * nu * ens) < 0.5


# Tier-1 struct conventions (vonkarman-diag/src/scalar.rs:22-54):
# enstrophy has no 1/2, edr = -2 nu Omega, cfl uses max|omega|.
def test_tier1_conventions_taylor_green():
    g = vo.Grid(16)
    s = vo.Periodic3D(g, 0.01, vo.taylor_green(g))
    d = s.tier1()
    assert abs(d["energy"] - 0.125) < 1e-12
    assert abs(d["enstrophy"] - 0.75) < 1e-12
    assert abs(d["energy_dissipation_rate"] + 2 * 0.01 * 0.75) < 1e-14
    assert abs(d["cfl_number"] - d["max_vorticity"] * d["dt"] / g.dx) < 1e-15


def test_cox_matthews_variant_is_fourth_order_on_linear_decay():
    # Pure viscous decay (N=0 mode): both variants are exact there, so check the
    # textbook variant converges at ~4th order against the reference variant on TG.
    g = vo.Grid(8)
    u0 = vo.taylor_green(g)
    errs = []
    ref = vo.Periodic3D(g, 0.05, u0, dt_mode="fixed", dt_fixed=0.0125, etd_variant="cox-matthews")
    for _ in range(16):
        ref.step()
    for dt in (0.1, 0.05):
        s = vo.Periodic3D(g, 0.05, u0, dt_mode="fixed", dt_fixed=dt, etd_variant="cox-matthews")
        for _ in range(int(round(0.2 / dt))):
            s.step()
        errs.append(max(np.abs(a - b).max() for a, b in zip(s.u_hat, ref.u_hat)))
    assert errs[1] < errs[0] / 8.0


# vonkarman-core/src/field.rs:147-199  grid_spec_basic / _spectral_shape / _padded / total_points
def test_grid_spec_basics():
    from vonkarman_gb300 import GridSpec
    g = vo.Grid(64)
    assert abs(g.dx - TWO_PI / 64) < 1e-14 and g.h == 33 and g.m == 96
    p = GridSpec(64)
    assert p.spectral_shape == (64, 64, 33) and abs(p.dx - TWO_PI / 64) < 1e-14
    assert p.padded_3half().n == 96
    assert GridSpec(32, 1.0).n ** 3 == 32 * 32 * 32


# vonkarman-periodic/src/ic/taylor_green.rs:45-52  taylor_green_divergence_free (w = 0)
def test_taylor_green_w_is_zero():
    from vonkarman_gb300 import ics
    assert np.abs(vo.taylor_green(vo.Grid(16))[2]).max() < 1e-14
    assert np.abs(ics.taylor_green(16)[2]).max() < 1e-14


# vonkarman-periodic/src/ic/abc.rs:49-64  abc_divergence_free (finite, w nonzero),
# :98-126  abc_is_beltrami (curl u = u, so <u . omega> = <|u|^2> = 2 E = 3)
def test_abc_finite_and_beltrami():
    g = vo.Grid(32)
    u = vo.abc_flow(g)
    phys = [vo.c2r_3d(c, (32, 32, 32)) for c in u]
    assert all(np.isfinite(p).all() for p in phys)
    assert np.abs(phys[2]).max() > 0.1
    s = vo.Periodic3D(g, 0.01, u)
    assert abs(s.energy() - 1.5) < 1e-6
    assert abs(s.helicity() - 3.0) < 1e-5


# vonkarman-diag/src/scalar.rs:61-86  diagnostics_from_zero_energy, energy_dissipation_identity
def test_scalar_diagnostics_zero_state_and_rates():
    from vonkarman_gb300.solver import ScalarDiagnostics
    rate, _ = ScalarDiagnostics.compute_rates(0.01, 10.0, 5.0)
    assert abs(rate - (-2.0 * 0.01 * 10.0)) < 1e-14
    g = vo.Grid(8)
    zero = [np.zeros((8, 8, 5), np.complex128) for _ in range(3)]
    d = vo.Periodic3D(g, 0.01, zero).tier1()
    assert d["energy"] == 0.0 and d["enstrophy"] == 0.0 and d["helicity"] == 0.0
    assert d["max_vorticity"] == 0.0 and d["energy_dissipation_rate"] == 0.0
