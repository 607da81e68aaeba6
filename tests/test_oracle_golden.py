"""CPU checks of the test infrastructure itself: the committed golden fixtures
reproduce from the numpy oracle, and the C restatement (the timed CPU
baseline) agrees with the numpy oracle."""

import math
import os

import numpy as np
import pytest

from oracle import vk_oracle as vo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def nrel(a, b):
    num = math.sqrt(sum(float(np.sum(np.abs(x - y) ** 2)) for x, y in zip(a, b)))
    den = math.sqrt(sum(float(np.sum(np.abs(y) ** 2)) for y in b))
    return num / den


def test_golden_fft_fixture_reproduces():
    z = np.load(os.path.join(GOLD, "fft_small.npz"))
    for i, shp in enumerate([(8, 8, 8), (12, 16, 24)]):
        assert np.abs(vo.r2c_3d(z[f"x{i}"]) - z[f"xh{i}"]).max() < 1e-13
        assert np.abs(vo.c2r_3d(z[f"yh{i}"], shp) - z[f"y{i}"]).max() < 1e-13


def test_golden_rand16_reproduces():
    z = np.load(os.path.join(GOLD, "rand16_cfl.npz"))
    g = vo.Grid(16)
    u0 = list(z["u0"])
    assert nrel(vo.compute_nonlinear(vo.SpectralOps(g), u0), list(z["nl0"])) < 1e-13
    s = vo.Periodic3D(g, float(z["nu"]), u0)
    assert abs(s.dt - float(z["dt0"])) < 1e-15
    s.step()
    assert nrel(s.u_hat, list(z["u1"])) < 1e-13


def test_golden_rand8_reproduces():
    z = np.load(os.path.join(GOLD, "rand8_fixed.npz"))
    g = vo.Grid(8)
    for name, kw in (("rk4", dict(integrator="rk4")), ("cm", dict(etd_variant="cox-matthews")), ("ref", {})):
        s = vo.Periodic3D(g, float(z["nu"]), list(z["u0"]), dt_mode="fixed", dt_fixed=float(z["dt"]), **kw)
        s.step()
        s.step()
        assert nrel(s.u_hat, list(z["u2_" + name])) < 1e-13


def test_golden_tg64_first_steps_reproduce():
    z = np.load(os.path.join(GOLD, "tg64_fixed.npz"))
    keys = list(z["keys"])
    g = vo.Grid(64)
    s = vo.Periodic3D(g, float(z["nu"]), vo.taylor_green(g), dt_mode="fixed", dt_fixed=float(z["dt"]))
    s.step()
    row = s.tier1()
    for j, k in enumerate(keys):
        ref = z["tier1"][1, j]
        assert abs(row[k] - ref) <= 1e-12 * max(abs(ref), 1e-300), k
    norms = np.array([np.sqrt(np.sum(np.abs(c) ** 2)) for c in s.u_hat])
    assert np.allclose(norms, z["norms_step1"], rtol=1e-13, atol=1e-300)


@pytest.fixture(scope="module")
def cpu():
    from oracle import vk_cpu

    vk_cpu.load()
    return vk_cpu


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 16, 24), (48, 32, 16), (96, 96, 96)])
def test_c_port_fft_matches_oracle(cpu, shape):
    rng = np.random.default_rng(5)
    x = rng.standard_normal(shape)
    xh = vo.r2c_3d(x)
    assert np.abs(cpu.r2c_3d(x) - xh).max() < 1e-12 * np.abs(xh).max()
    yh = xh + 0.2j * rng.standard_normal(xh.shape)
    y = vo.c2r_3d(yh, shape)
    assert np.abs(cpu.c2r_3d(yh, shape) - y).max() < 1e-12 * np.abs(y).max()


@pytest.mark.parametrize("n", [8, 16, 32])
def test_c_port_nonlinear_and_steps_match_oracle(cpu, n):
    g = vo.Grid(n)
    u = vo.hermitian_clean(g, vo.random_field(g, n, amp=float(n) ** 3 / 30.0))
    s = cpu.CpuSolver(n, 0.01, u)
    assert nrel(s.nonlinear(u), vo.compute_nonlinear(vo.SpectralOps(g), u)) < 1e-13
    o = vo.Periodic3D(g, 0.01, u)
    assert abs(s.dt() - o.dt) <= 1e-14 * o.dt
    s.step(3)
    for _ in range(3):
        o.step()
    assert nrel(s.u_hat(), o.u_hat) < 1e-13
    assert abs(s.time() - o.time) <= 1e-14 * o.time


def test_c_restatement_spectrum_vs_numpy_oracle():
    """vkc_spectrum (energy_spectrum, spectrum.rs:13-60, in the C restatement
    the reference arm of bench.py times) against the numpy oracle."""
    from oracle import vk_cpu

    n = 32
    g = vo.Grid(n, 3.0)
    u = vo.hermitian_clean(g, vo.random_field(g, 8, amp=100.0))
    c = vk_cpu.CpuSolver(n, 0.01, u, l=3.0)
    got = c.spectrum()
    c.close()
    _, want = vo.energy_spectrum(u, vo.SpectralOps(g))
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
