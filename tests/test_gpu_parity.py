"""GPU parity: the CUDA path (through the C ABI) against the numpy oracle on
the same inputs.  FP64 comparisons bound two errors: norm-relative
||a - b||_2 / ||b||_2 over all components, and per coefficient
max |a - b| / max |b| (element-wise relative error is ill-posed for the ~0
modes; the max-coefficient form still sees a large error on a few modes).

Tolerances (FP64): 1e-12 for spectral coefficients after one step or one
nonlinear evaluation, 1e-10 for Tier-1 diagnostics and E(k); FP32-bulk: 2e-5
(one step) against the FP64 oracle.
"""

import math

import numpy as np
import pytest

from oracle import vk_oracle as vo

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_DIAG = 1e-10
TOL32 = 2e-5


def nrel(a, b):
    num = math.sqrt(sum(float(np.sum(np.abs(x - y) ** 2)) for x, y in zip(a, b)))
    den = math.sqrt(sum(float(np.sum(np.abs(y) ** 2)) for y in b))
    return num / den if den > 0 else num


def maxcoef(a, b):
    """max |a - b| / max |b| over all coefficients of all components: a large
    error on a few small coefficients cannot hide behind the norm."""
    num = max(float(np.max(np.abs(x - y))) for x, y in zip(a, b))
    den = max(float(np.max(np.abs(y))) for y in b)
    return num / den if den > 0 else num


def close(a, b, tol):
    """Both metrics within tol."""
    e1, e2 = nrel(a, b), maxcoef(a, b)
    assert e1 < tol and e2 < tol, (e1, e2, tol)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def vk():
    import vonkarman_gb300 as vk

    return vk


def random_state(n, seed, clean=True):
    g = vo.Grid(n)
    u = vo.random_field(g, seed)
    if clean:
        u = vo.hermitian_clean(g, u)
    return u


# --- FftBackend contract (backend.rs:9-25; ndrustfft_backend.rs:75-147) -----

@pytest.mark.parametrize("shape", [(8, 8, 8), (16, 16, 16), (32, 32, 32), (64, 64, 64), (12, 12, 12),
                                   (24, 24, 24), (96, 96, 96), (16, 24, 32), (48, 8, 12), (128, 128, 128)])
def test_fft_r2c_c2r_vs_numpy(vk, shape):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    f = vk.GpuFftBackend(*shape)
    xh = f.r2c_3d(x)
    ref = np.fft.rfftn(x)
    close([xh], [ref], TOL64)
    back = f.c2r_3d(xh)
    assert np.abs(back - x).max() < 1e-12 * max(1.0, np.abs(x).max())
    # c2r of a non-Hermitian input: imaginary parts of DC/Nyquist planes ignored
    yh = ref + 0.3j * rng.standard_normal(ref.shape)
    got = f.c2r_3d(yh)
    want = np.fft.irfftn(yh, s=shape, axes=(0, 1, 2))
    assert np.abs(got - want).max() < 1e-12 * np.abs(want).max()
    f.close()


# Every line length of the x / y passes (register-resident engine) and of the
# z passes, in both precision forms: the 3/2-padded lengths up to M = 768
# (N = 512) and the N-grid lengths up to 512.
@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32bulk", 1e-6)])
@pytest.mark.parametrize("shape", [(768, 384, 8), (512, 256, 8), (192, 128, 8), (96, 48, 16), (32, 24, 12),
                                   (16, 12, 8), (8, 64, 8), (8, 8, 768), (8, 8, 384), (8, 16, 512)])
def test_fft_all_line_lengths_vs_numpy(vk, precision, tol, shape):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape)
    f = vk.GpuFftBackend(*shape, precision=precision)
    ref = np.fft.rfftn(x)
    xh = f.r2c_3d(x)
    assert nrel([xh], [ref]) < tol
    if precision == "fp64":
        assert maxcoef([xh], [ref]) < tol
    assert np.abs(f.c2r_3d(ref) - x).max() < 100 * tol * max(1.0, np.abs(x).max())
    f.close()


def test_fft_roundtrip_and_parseval_kats(vk):
    # ndrustfft_backend.rs:75-106 (roundtrip 1e-12) and :108-147 (Parseval 1e-10)
    n = 8
    x = np.sin(2 * np.pi * np.arange(n) / n)[:, None, None] * np.ones((n, n, n))
    f = vk.GpuFftBackend(n, n, n)
    assert np.abs(f.c2r_3d(f.r2c_3d(x)) - x).max() < 1e-12
    n = 16
    i = np.arange(n)
    x = (np.sin(2 * np.pi * i / n)[:, None, None] + np.cos(2 * np.pi * i / n)[None, :, None]) * np.ones((n, n, n))
    f = vk.GpuFftBackend(n, n, n)
    s = f.r2c_3d(x)
    w = np.full(n // 2 + 1, 2.0)
    w[0] = w[-1] = 1.0
    spec = float((w * np.abs(s) ** 2).sum()) / n ** 3
    assert abs(float((x * x).sum()) - spec) / float((x * x).sum()) < 1e-10
    assert f.name() and f.precision_digits() == 15


def test_fft_fp32_backend(vk):
    rng = np.random.default_rng(2)
    x = rng.standard_normal((64, 64, 64))
    f = vk.GpuFftBackend(64, 64, 64, precision="fp32bulk")
    assert nrel([f.r2c_3d(x)], [np.fft.rfftn(x)]) < 1e-6
    assert f.precision_digits() == 6


# --- compute_nonlinear (nonlinear.rs:15-39, dealiased.rs:16-110) -------------

@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_nonlinear_vs_oracle(vk, n):
    g = vo.Grid(n)
    u = random_state(n, 10 + n)
    want = vo.compute_nonlinear(vo.SpectralOps(g), u)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u, vk.SolverOptions(dt_mode="fixed", dt_fixed=1e-3))
    got = vk.compute_nonlinear(s, u)
    close(got, want, TOL64)
    s.close()


@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32bulk", TOL32)])
def test_nonlinear_vs_oracle_n128(vk, precision, tol):
    n = 128
    g = vo.Grid(n)
    u = random_state(n, 7)
    want = vo.compute_nonlinear(vo.SpectralOps(g), u)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u, vk.SolverOptions(precision=precision, dt_mode="fixed",
                                                                   dt_fixed=1e-3))
    got = vk.compute_nonlinear(s, u)
    assert nrel(got, want) < tol
    if precision == "fp64":
        assert maxcoef(got, want) < tol
    s.close()


def test_nonlinear_fp32bulk_vs_fp64_n256(vk):
    # M = 384 plans of both forms against each other (the oracle is too slow
    # at this size): agreement to the FP32 level
    from vonkarman_gb300 import ics

    n = 256
    u = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=5)
    out = []
    for prec in ("fp64", "fp32bulk"):
        s = vk.Periodic3D(vk.GridSpec(n), 1e-3, u, vk.SolverOptions(precision=prec, dt_mode="fixed",
                                                                      dt_fixed=1e-3))
        out.append(vk.compute_nonlinear(s, u))
        s.close()
    assert nrel(out[1], out[0]) < TOL32


def test_nonlinear_fp32bulk_vs_fp64_n512(vk):
    # the 768-point plans of both forms (one column pair per CTA, z pass in
    # place) against each other: agreement to the FP32 level
    from vonkarman_gb300 import ics

    n = 512
    u = ics.lamb_oseen_tubes(n)
    out = []
    for prec in ("fp64", "fp32bulk"):
        s = vk.Periodic3D(vk.GridSpec(n), 5e-4, u, vk.SolverOptions(precision=prec, dt_mode="fixed",
                                                                      dt_fixed=1e-3))
        out.append(vk.compute_nonlinear(s, u))
        s.close()
    assert nrel(out[1], out[0]) < TOL32


def test_nonlinear_non_hermitian_input(vk):
    # raw random spectral data (not Hermitian in the kz=0 plane): the padded
    # c2r must drop exactly what the reference's backend drops
    n = 16
    g = vo.Grid(n)
    u = random_state(n, 7, clean=False)
    want = vo.compute_nonlinear(vo.SpectralOps(g), u)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u, vk.SolverOptions(dt_mode="fixed", dt_fixed=1e-3))
    close(vk.compute_nonlinear(s, u), want, TOL64)


def test_nonlinear_divergence_free_kat(vk):
    # nonlinear.rs:50-97: |k . N_hat| < 1e-6 for Taylor-Green at N=16
    n = 16
    g = vo.Grid(n)
    ops = vo.SpectralOps(g)
    u = vo.taylor_green(g)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u)
    nl = vk.compute_nonlinear(s, u)
    div = ops.KX * nl[0] + ops.KY * nl[1] + ops.KZ * nl[2]
    assert np.abs(div).max() < 1e-6


def test_dealiased_zero_and_antisymmetry_kats(vk):
    # dealiased.rs:173-202 (zero in -> zero out).  The anti-symmetry KAT
    # (:204-263) is a property of the cross product itself; here the same
    # P1..P5 chain is checked against the oracle for a single-mode state.
    n = 8
    g = vo.Grid(n)
    z = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, z, vk.SolverOptions(dt_mode="fixed", dt_fixed=1e-3))
    for c in vk.compute_nonlinear(s, z):
        assert np.abs(c).max() < 1e-14
    u = [np.zeros(g.spectral_shape, complex) for _ in range(3)]
    u[0][1, 2, 1] = 3.0 + 1.0j
    u[1][n - 2, 1, 3] = -2.0 + 0.5j
    u[2][3, n - 1, 4] = 1.5 - 0.7j  # z-Nyquist plane (iz = n/2)
    want = vo.compute_nonlinear(vo.SpectralOps(g), u)
    close(vk.compute_nonlinear(s, u), want, TOL64)


# --- one step / many steps ---------------------------------------------------

def test_one_step_taylor_green_n64_fixed_dt(vk):
    # the CPU-runnable Taylor-Green case: N=64, nu=6.25e-4, fixed dt=1e-3
    n, nu, dt = 64, 6.25e-4, 1e-3
    g = vo.Grid(n)
    u0 = vo.taylor_green(g)
    ref = vo.Periodic3D(g, nu, u0, dt_mode="fixed", dt_fixed=dt)
    ref.step()
    s = vk.Periodic3D(vk.GridSpec(n), nu, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=dt))
    s.step()
    close(s.u_hat(), ref.u_hat, TOL64)
    assert s.time() == pytest.approx(dt, rel=0, abs=0)


def test_taylor_green_n64_100_steps_tier1_and_spectrum_vs_golden(vk):
    # the CPU-runnable Taylor-Green case over its 100 steps: Tier-1 after every
    # step within 1e-10 relative, E(k) at step 100 (golden fixture made by the
    # oracle, tests/golden/make_golden.py)
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "tg64_fixed.npz"))
    n, nu, dt = int(z["n"]), float(z["nu"]), float(z["dt"])
    keys = [str(k) for k in z["keys"]]
    s = vk.Periodic3D(vk.GridSpec(n), nu, vo.taylor_green(vo.Grid(n)),
                      vk.SolverOptions(dt_mode="fixed", dt_fixed=dt))
    recs = s.run(100, every=1)
    assert len(recs) == 100
    scale = float(z["tier1"][0, keys.index("enstrophy")])
    for i, r in enumerate(recs):
        for j, k in enumerate(keys):
            ref = float(z["tier1"][i + 1, j])
            got = float(getattr(r, k))
            # helicity-type values of Taylor-Green are zero up to rounding: an
            # absolute floor of 1e-10 x the enstrophy scale
            tol = max(TOL_DIAG * abs(ref), TOL_DIAG * scale if "helicity" in k else 0.0)
            assert abs(got - ref) <= tol, (i + 1, k, got, ref)
    shells, spec = vk.energy_spectrum(s)
    assert np.array_equal(shells, z["shells"])
    assert np.abs(spec - z["spectrum"]).max() <= TOL_DIAG * np.abs(z["spectrum"]).max()


@pytest.mark.parametrize("n", [16, 32])
def test_steps_random_cfl_vs_oracle(vk, n):
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 3, amp=float(n) ** 3 / 40.0))
    nu = 0.02
    ref = vo.Periodic3D(g, nu, u0)
    s = vk.Periodic3D(vk.GridSpec(n), nu, u0)
    assert rel(s.dt(), ref.dt) < 1e-13
    for _ in range(5):
        ref.step()
    s.step(5)
    close(s.u_hat(), ref.u_hat, 1e-11)
    assert rel(s.dt(), ref.dt) < 1e-12
    assert rel(s.time(), ref.time) < 1e-12
    assert s.step_count() == 5


@pytest.mark.parametrize("variant", ["reference", "cox-matthews"])
def test_etd_variants_vs_oracle(vk, variant):
    n = 16
    g = vo.Grid(n)
    u0 = vo.taylor_green(g)
    ref = vo.Periodic3D(g, 0.05, u0, dt_mode="fixed", dt_fixed=0.01, etd_variant=variant)
    s = vk.Periodic3D(vk.GridSpec(n), 0.05, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=0.01,
                                                                   etd_variant=variant))
    for _ in range(3):
        ref.step()
    s.step(3)
    close(s.u_hat(), ref.u_hat, TOL64)


def test_rk4_vs_oracle(vk):
    n = 16
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 5, amp=50.0))
    ref = vo.Periodic3D(g, 0.01, u0, dt_mode="fixed", dt_fixed=1e-3, integrator="rk4")
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, vk.SolverOptions(dt_mode="fixed", dt_fixed=1e-3,
                                                                   integrator="rk4"))
    for _ in range(3):
        ref.step()
    s.step(3)
    close(s.u_hat(), ref.u_hat, TOL64)


def test_tier1_and_spectrum_vs_oracle(vk):
    n = 32
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 9, amp=200.0))
    ref = vo.Periodic3D(g, 0.01, u0)
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0)
    for _ in range(3):
        ref.step()
    s.step(3)
    want = ref.tier1()
    got = s.tier1()
    for k, v in want.items():
        if k == "step":
            assert got.step == v
            continue
        tol = TOL_DIAG if k != "helicity" else 1e-9
        assert abs(getattr(got, k) - v) <= tol * max(abs(v), 1e-300) + 1e-13, k
    shells, spec = vk.energy_spectrum(s)
    sh_ref, spec_ref = vo.energy_spectrum(ref.u_hat, ref.ops)
    assert np.array_equal(shells, sh_ref)
    assert np.abs(spec - spec_ref).max() <= TOL_DIAG * np.abs(spec_ref).max()
    assert s.cfl_dt() == pytest.approx(ref.compute_cfl_dt(), rel=1e-13)


@pytest.mark.parametrize("n,l,prec", [(32, 3.0, "fp64"), (64, 2.0 * math.pi, "fp32bulk"), (64, 5.0, "fp32bulk")])
def test_tier1_and_spectrum_box_lengths_and_precisions(vk, n, l, prec):
    """Diagnostics of the initial state against the oracle, on boxes whose
    wavenumber scale is not 1 (shells from the FP64 |k| path) and in the
    FP32-bulk form (per-mode products in FP32, FP64 sums).  Helicity and
    superhelicity can cancel far below their bounds, so their error is
    measured against sqrt(E Omega) and kmax Omega."""
    g = vo.Grid(n, l)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 11, amp=200.0))
    ref = vo.Periodic3D(g, 0.01, u0)
    s = vk.Periodic3D(vk.GridSpec(n, l), 0.01, u0, vk.SolverOptions(precision=prec))
    want = ref.tier1()
    got = s.tier1()
    tol = TOL_DIAG if prec == "fp64" else 1e-6
    kmax = (2.0 * math.pi / l) * (n // 2)
    scale = {"helicity": math.sqrt(want["energy"] * want["enstrophy"]),
             "superhelicity": kmax * want["enstrophy"],
             "helicity_dissipation_rate": 2.0 * 0.01 * kmax * want["enstrophy"]}
    for k in ("energy", "enstrophy", "helicity", "superhelicity", "max_vorticity", "energy_dissipation_rate",
              "helicity_dissipation_rate", "cfl_number"):
        v = want[k]
        assert abs(getattr(got, k) - v) <= tol * max(abs(v), scale.get(k, 0.0)), (k, getattr(got, k), v)
    shells, spec = vk.energy_spectrum(s)
    sh_ref, spec_ref = vo.energy_spectrum(ref.u_hat, ref.ops)
    assert np.array_equal(shells, sh_ref)
    assert np.abs(spec - spec_ref).max() <= tol * np.abs(spec_ref).max()


def test_restart_bitwise(vk):
    # solver.rs:673-706 / tests/checkpoint_restart.rs:10-63
    n = 16
    g = vo.Grid(n)
    u0 = vo.taylor_green(g)
    cont = vk.Periodic3D(vk.GridSpec(n), 0.01, u0)
    cont.step(20)
    half = vk.Periodic3D(vk.GridSpec(n), 0.01, u0)
    half.step(10)
    rest = vk.Periodic3D.from_checkpoint(half.checkpoint_data())
    rest.step(10)
    for a, b in zip(cont.u_hat(), rest.u_hat()):
        assert np.array_equal(a, b)
    assert cont.time() == rest.time() and cont.step_count() == rest.step_count()


def test_run_records_match_tier1(vk):
    """vk_run's records (Tier-1 sums fused into the final stage of each record
    step) against vk_tier1's separate pass over the same states: the same
    per-mode terms summed in another order, so equal to rounding; the state,
    time, dt and max|omega| are bitwise equal."""
    n = 16
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 6, amp=200.0))
    a = vk.Periodic3D(vk.GridSpec(n), 0.01, u0)
    recs = a.run(6, every=2)
    b = vk.Periodic3D(vk.GridSpec(n), 0.01, u0)
    for r in recs:
        b.step(2)
        t = b.tier1()
        assert r.step == t.step
        for k in ("time", "dt", "max_vorticity"):
            assert getattr(r, k) == getattr(t, k), k
        for k in ("energy", "enstrophy", "helicity", "superhelicity"):
            scale = math.sqrt(t.energy * t.enstrophy) if "helicity" in k else abs(getattr(t, k))
            assert abs(getattr(r, k) - getattr(t, k)) <= 1e-13 * max(scale, 1e-300), k
    assert all(np.array_equal(x, y) for x, y in zip(a.u_hat(), b.u_hat()))


@pytest.mark.parametrize("precision,n", [("fp64", 32), ("fp32bulk", 32), ("fp32bulk", 64)])
def test_fused_diagnostics_match_separate_passes(vk, precision, n):
    """Tier-1 sums and E(k) accumulated inside the final stage of a step
    (vk_set_fused_diagnostics) against the separate reduction passes over the
    same state: equal to rounding of the FP64 sums."""
    g = vo.Grid(n, 2.0 * math.pi if n == 64 else 3.0)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 14, amp=float(n) ** 3 / 30.0))
    opts = vk.SolverOptions(precision=precision)
    a = vk.Periodic3D(vk.GridSpec(n, g.l), 0.01, u0, opts)
    b = vk.Periodic3D(vk.GridSpec(n, g.l), 0.01, u0, opts)
    a.set_fused_diagnostics(1, 2)
    for step in range(1, 5):
        a.step(1)
        b.step(1)
        ta, tb = a.tier1(), b.tier1()
        for k in ("energy", "enstrophy", "helicity", "superhelicity", "max_vorticity"):
            scale = math.sqrt(tb.energy * tb.enstrophy) if "helicity" in k else abs(getattr(tb, k))
            assert abs(getattr(ta, k) - getattr(tb, k)) <= 1e-13 * scale, (step, k)
        sa, sb = vk.energy_spectrum(a)[1], vk.energy_spectrum(b)[1]
        assert np.abs(sa - sb).max() <= 1e-13 * sb.max(), step
    assert all(np.array_equal(x, y) for x, y in zip(a.u_hat(), b.u_hat()))
    a.close()
    b.close()


@pytest.mark.parametrize("integrator,variant", [("rk4", "reference"), ("etd-rk4", "cox-matthews")])
def test_fp32bulk_one_step_other_integrators(vk, integrator, variant):
    # the RK4 and Cox-Matthews stage epilogues in the FP32-bulk form
    n = 32
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 4, amp=100.0))
    ref = vo.Periodic3D(g, 0.01, u0, dt_mode="fixed", dt_fixed=2e-3, integrator=integrator, etd_variant=variant)
    ref.step()
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, vk.SolverOptions(precision="fp32bulk", dt_mode="fixed",
                                                                   dt_fixed=2e-3, integrator=integrator,
                                                                   etd_variant=variant))
    s.step()
    assert nrel(s.u_hat(), ref.u_hat) < TOL32


def test_fp32bulk_one_step(vk):
    n = 32
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 4, amp=100.0))
    ref = vo.Periodic3D(g, 0.01, u0, dt_mode="fixed", dt_fixed=2e-3)
    ref.step()
    s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, vk.SolverOptions(precision="fp32bulk", dt_mode="fixed",
                                                                   dt_fixed=2e-3))
    s.step()
    assert nrel(s.u_hat(), ref.u_hat) < TOL32
    e = s.energy()
    assert rel(e, ref.energy()) < 1e-6


@pytest.mark.parametrize("precision,integrator", [("fp64", "etd-rk4"), ("fp32bulk", "etd-rk4"), ("fp64", "rk4")])
def test_graph_replay_matches_eager_launches(vk, precision, integrator):
    """Steps replayed as captured CUDA graphs (the default) against eager
    launches: bitwise equal states, time and Tier-1 records, with the fused
    diagnostics cadence changing the launch sequence between steps."""
    n = 32
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 17, amp=float(n) ** 3 / 40.0))
    opts = vk.SolverOptions(precision=precision, integrator=integrator)
    runs = []
    for graphs in (True, False):
        s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, opts)
        s.use_graphs(graphs)
        s.set_fused_diagnostics(3, 4)
        s.step(7)
        recs = s.run(6, every=2)
        s.step(5)
        runs.append((s.u_hat(), s.time(), s.dt(), [(r.energy, r.enstrophy, r.max_vorticity) for r in recs]))
        s.close()
    (ua, ta, da, ra), (ub, tb, db, rb) = runs
    assert all(np.array_equal(x, y) for x, y in zip(ua, ub))
    assert ta == tb and da == db and ra == rb
