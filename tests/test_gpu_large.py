"""FP64 parity at the grids the benchmark and the target workload run: one
ETD-RK4 step (adaptive CFL dt, ETD tabulation, four nonlinear evaluations
with the 384- and 768-point padded plans) of the GPU against the oracle's C
restatement of the reference CPU path (oracle/vk_cpu.c, all host cores) on
the same initial state, then Tier-1 and E(k) of the GPU state against the
numpy oracle's diagnostics of the C restatement's state.

Tolerances: 1e-12 for the spectral state both norm-relative
(||a - b|| / ||b||) and per coefficient (max |a - b| / max |b|, which a
large error on a few small coefficients cannot hide behind); 1e-12 for dt
and time; 1e-10 for every Tier-1 value (helicity-type values against the
bounds sqrt(E Omega) and kmax Omega, as they can cancel) and for E(k)
relative to its largest shell.
"""

import math
import os

import numpy as np
import pytest

from oracle import vk_oracle as vo

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_DIAG = 1e-10


def nrel(a, b):
    num = math.sqrt(sum(float(np.sum(np.abs(x - y) ** 2)) for x, y in zip(a, b)))
    den = math.sqrt(sum(float(np.sum(np.abs(y) ** 2)) for y in b))
    return num / den


def maxcoef(a, b):
    num = max(float(np.max(np.abs(x - y))) for x, y in zip(a, b))
    den = max(float(np.max(np.abs(y))) for y in b)
    return num / den


def host_mem_available_gb() -> float:
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 2 ** 20
    except OSError:
        pass
    return 0.0


CASES = {
    # the benchmark workload: random isotropic, von Karman kp=4, E=0.5, seed 42
    256: dict(nu=1e-3, ic="isotropic", host_gb=40.0),
    # the target workload: anti-parallel Lamb-Oseen tubes
    512: dict(nu=5e-4, ic="tubes", host_gb=120.0),
}


@pytest.mark.parametrize("n", [256, 512])
def test_one_step_fp64_vs_c_restatement(n):
    import vonkarman_gb300 as vk
    from oracle import vk_cpu
    from vonkarman_gb300 import ics

    case = CASES[n]
    avail = host_mem_available_gb()
    if avail < case["host_gb"]:
        pytest.skip(f"host RAM: the C restatement of the reference dataflow at N={n} needs about "
                    f"{case['host_gb']:.0f} GB, {avail:.0f} GB available")
    u0 = (ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=42) if case["ic"] == "isotropic"
          else ics.lamb_oseen_tubes(n))
    nu = case["nu"]

    s = vk.Periodic3D(vk.GridSpec(n), nu, u0)
    dt0 = s.dt()
    s.step(1)
    got = s.u_hat()
    t1 = s.tier1()
    _, spec = vk.energy_spectrum(s)
    dt_gpu, time_gpu = s.dt(), s.time()
    s.close()

    vk_cpu.set_threads(len(os.sched_getaffinity(0)))
    c = vk_cpu.CpuSolver(n, nu, u0)
    dt0_cpu = c.dt()
    c.step(1)
    want = c.u_hat()
    dt_cpu, time_cpu = c.dt(), c.time()
    c.close()

    assert abs(dt0 - dt0_cpu) <= TOL64 * dt0_cpu
    assert abs(dt_gpu - dt_cpu) <= TOL64 * dt_cpu
    assert abs(time_gpu - time_cpu) <= TOL64 * time_cpu
    e_norm, e_max = nrel(got, want), maxcoef(got, want)
    print(f"N={n}: state norm-rel {e_norm:.2e}, max-coef {e_max:.2e}")
    assert e_norm < TOL64
    assert e_max < TOL64

    g = vo.Grid(n)
    ref = vo.tier1_of_state(g, nu, want, time_cpu, 1, dt_cpu)
    kmax = n // 2
    scale = {"helicity": math.sqrt(ref["energy"] * ref["enstrophy"]),
             "superhelicity": kmax * ref["enstrophy"],
             "helicity_dissipation_rate": 2.0 * nu * kmax * ref["enstrophy"]}
    for k in ("energy", "enstrophy", "helicity", "superhelicity", "max_vorticity", "energy_dissipation_rate",
              "helicity_dissipation_rate", "cfl_number", "dt", "time"):
        v = ref[k]
        assert abs(getattr(t1, k) - v) <= TOL_DIAG * max(abs(v), scale.get(k, 0.0)), (k, getattr(t1, k), v)
    assert t1.step == 1
    _, spec_ref = vo.energy_spectrum(want, vo.SpectralOps(g))
    assert np.abs(spec - spec_ref).max() <= TOL_DIAG * np.abs(spec_ref).max()


def test_reference_cufft_mode_matches_cpu_mode():
    """The reference's cuFFT GPU mode as restated for the timed baseline
    (oracle/vk_cpu.c with vkc_set_cufft: per-call copies around cuFFT, host
    normalisation, vonkarman-fft/src/cufft.rs:249-319) takes the same step as
    the CPU mode to FFT rounding."""
    from oracle import vk_cpu

    n, nu = 32, 0.02
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 3, amp=float(n) ** 3 / 40.0))
    cpu = vk_cpu.CpuSolver(n, nu, u0)
    cpu.step(2)
    vk_cpu.set_cufft(True)
    try:
        gpu = vk_cpu.CpuSolver(n, nu, u0)
        assert gpu.uses_cufft()
        gpu.step(2)
        got = gpu.u_hat()
        gpu.close()
    finally:
        vk_cpu.set_cufft(False)
    want = cpu.u_hat()
    assert nrel(got, want) < 1e-12
    cpu.close()


@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32bulk", 2e-5)])
def test_nonlinear_n256_vs_c_restatement(precision, tol):
    """compute_nonlinear at N=256 (384-point padded plans; in FP32-bulk the
    fused z-pass kernel) against the C restatement of the reference's
    dealiased product (oracle/vk_cpu.c): FP64 to 1e-12 in both metrics,
    FP32-bulk to its 2e-5 norm-relative bound."""
    import vonkarman_gb300 as vk
    from oracle import vk_cpu
    from vonkarman_gb300 import ics

    n = 256
    u = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=9)
    vk_cpu.set_threads(len(os.sched_getaffinity(0)))
    c = vk_cpu.CpuSolver(n, 1e-3, u, dt_mode="fixed", dt_fixed=1e-3)
    want = c.nonlinear(u)
    c.close()
    s = vk.Periodic3D(vk.GridSpec(n), 1e-3, u, vk.SolverOptions(precision=precision, dt_mode="fixed",
                                                                   dt_fixed=1e-3))
    got = vk.compute_nonlinear(s, u)
    s.close()
    e_norm, e_max = nrel(got, want), maxcoef(got, want)
    print(f"{precision}: norm-rel {e_norm:.2e}, max-coef {e_max:.2e}")
    assert e_norm < tol
    if precision == "fp64":
        assert e_max < tol
