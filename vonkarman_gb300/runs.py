"""Run loop and the long workloads of the periodic step.

``run_to_time`` is the time loop of vonkarman-bin (run.rs:107-182: step, then
Tier-1 diagnostics, stop at the first step whose time reaches ``max_time``)
with the diagnostics recorded on the device by ``vk_run`` and read back once
per chunk instead of once per step.

Workloads run from here (``python -m vonkarman_gb300.runs <name>``):

* ``tg``     -- Taylor-Green N=64, nu = 6.25e-4, fixed dt = 1e-3, 100 steps,
  Tier-1 after every step, E(k) at step 100 (FP64): steps/s with the
  diagnostics and device-timed steps/s without them.
* ``isotropic`` -- random isotropic (von Karman kp = 4, E = 0.5, seed 42)
  N=256, nu = 1e-3, adaptive CFL 0.5, to t = 2, Tier-1 after every step and
  E(k) every 10 steps, FP64 and FP32-bulk: steps/s with the diagnostics, and
  the FP32-bulk error against FP64 at t = 2.
* ``tubes``  -- anti-parallel Lamb-Oseen tubes (circulation +-1, core radius
  0.25, separation 1.0 about (pi, pi), centre lines displaced in x by
  0.1 sin z), nu = 5e-4, adaptive CFL 0.5, to t = 5, Tier-1 after every step,
  FP32-bulk against FP64: steps/s of both forms and the relative error of the
  energy, enstrophy and max|omega| at t = 5.
* ``ascent`` -- random isotropic start (kp = 3, E = 0.5), nu = 2e-3, fixed
  dt = 1e-3, 1000 steps, 20 level-1 checkpoints: the FP32-bulk and FP64
  gradients of the final enstrophy, the adjoint/forward cost ratio of both
  forms, the FP32-bulk gradient error against the FP64 one, and 10
  projected-gradient ascent iterations on the sphere <u, u> = 1.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import ics, optimize
from .solver import GridSpec, Periodic3D, SolverOptions, l2_inner


def run_to_time(solver: Periodic3D, t_end: float, every: int = 1, max_chunk: int = 200):
    """Step until ``solver.time() >= t_end`` (the stop rule of run.rs:152-155)
    and return the Tier-1 records of every ``every``-th step.  Chunks are sized
    from the current dt so that the loop does not pass the first step that
    reaches ``t_end``; the last few steps are taken one at a time (with
    ``every`` > 1 chunks are multiples of ``every``, so the run may end up to
    ``every`` - 1 steps past that step)."""
    recs = []
    while solver.time() < t_end:
        dt = solver.dt()
        left = t_end - solver.time()
        k = int(0.9 * left / dt) if dt > 0 else 1
        k = max(1, min(max_chunk, k))
        if every > 1:
            k = max(every, k - k % every)
        recs.extend(solver.run(k, every))
    return recs


def interp_at(recs, t: float, name: str) -> float:
    """Linear interpolation of a Tier-1 field at time t between the records
    that bracket it."""
    ts = np.array([r.time for r in recs])
    vs = np.array([getattr(r, name) for r in recs])
    return float(np.interp(t, ts, vs))


def _timed_rate(solver: Periodic3D, steps: int) -> float:
    solver.step(3)
    ms = solver.step_timed(steps)
    return 1000.0 * steps / ms


def run_to_time_spectra(solver: Periodic3D, t_end: float, max_chunk: int = 200):
    """``run_to_time`` with Tier-1 after every step, plus the shell spectrum of
    the last state before ``t_end`` and of the first state at or past it, so
    that E(k) can be interpolated to ``t_end`` like the Tier-1 series.
    Returns (records, (t_a, E_a), (t_b, E_b))."""
    from .solver import energy_spectrum

    recs = []
    while True:
        dt = solver.dt()
        left = t_end - solver.time()
        k = int(0.9 * left / dt) - 1 if dt > 0 else 0
        if k < 2:
            break
        recs.extend(solver.run(min(max_chunk, k), 1))
    before = (solver.time(), energy_spectrum(solver)[1])
    while solver.time() < t_end:
        before = (solver.time(), energy_spectrum(solver)[1])
        recs.extend(solver.run(1, 1))
    after = (solver.time(), energy_spectrum(solver)[1])
    return recs, before, after


def _interp_spec(a, b, t):
    (ta, ea), (tb, eb) = a, b
    if tb <= ta:
        return eb
    f = (t - ta) / (tb - ta)
    return (1.0 - f) * ea + f * eb


def tubes(n: int = 512, nu: float = 5e-4, t_end: float = 5.0, rate_steps: int = 20, device: int = 0) -> dict:
    grid = GridSpec(n)
    u0 = ics.lamb_oseen_tubes(n, circulation=1.0, sigma=0.25, separation=1.0, eps=0.1)
    out = {"workload": f"anti-parallel Lamb-Oseen tubes N={n}, nu={nu}, adaptive CFL 0.5, to t={t_end}, "
                       "Tier-1 after every step", "forms": {}}
    series, spec_end = {}, {}
    for prec in ("fp64", "fp32bulk"):
        s = Periodic3D(grid, nu, u0, SolverOptions(precision=prec, device=device))
        t0 = time.perf_counter()
        recs, sa, sb = run_to_time_spectra(s, t_end)
        wall = time.perf_counter() - t0
        series[prec] = recs
        spec_end[prec] = _interp_spec(sa, sb, t_end)
        u_end = s.u_hat() if prec == "fp64" else None
        rate = _timed_rate(s, rate_steps)
        out["forms"][prec] = {"steps": len(recs), "t_last": recs[-1].time, "wall_s": wall,
                              "steps_per_s_with_tier1": len(recs) / wall,
                              "steps_per_s": rate,
                              "energy_t_end": interp_at(recs, t_end, "energy"),
                              "enstrophy_t_end": interp_at(recs, t_end, "enstrophy"),
                              "max_vorticity_t_end": interp_at(recs, t_end, "max_vorticity")}
        s.close()
        del u_end
    f64, f32 = out["forms"]["fp64"], out["forms"]["fp32bulk"]
    out["speedup_fp32bulk_over_fp64"] = f32["steps_per_s"] / f64["steps_per_s"]
    out["rel_error_at_t_end"] = {k: abs(f32[k + "_t_end"] - f64[k + "_t_end"]) / abs(f64[k + "_t_end"])
                                 for k in ("energy", "enstrophy", "max_vorticity")}
    a, b = spec_end["fp64"], spec_end["fp32bulk"]
    keep = a > 1e-12 * a.max()
    out["rel_error_at_t_end"]["spectrum_max_rel_shell"] = float(np.max(np.abs(b - a)[keep] / a[keep]))
    out["rel_error_at_t_end"]["spectrum_max_abs_over_max"] = float(np.max(np.abs(b - a)) / a.max())
    # the largest relative deviation over the run, at equal times
    a, b = series["fp64"], series["fp32bulk"]
    tt = np.array([r.time for r in a])
    tt = tt[tt <= min(a[-1].time, b[-1].time)]
    worst = {}
    for k in ("energy", "enstrophy", "max_vorticity"):
        va = np.interp(tt, [r.time for r in a], [getattr(r, k) for r in a])
        vb = np.interp(tt, [r.time for r in b], [getattr(r, k) for r in b])
        worst[k] = float(np.max(np.abs(vb - va) / np.abs(va)))
    out["max_rel_deviation_over_run"] = worst
    return out


def tg(n: int = 64, nu: float = 6.25e-4, dt: float = 1e-3, steps: int = 100, device: int = 0) -> dict:
    """Both forms; the FP32-bulk form's error against the FP64 run after the
    last step (E, enstrophy, max|omega|, per-shell E(k))."""
    from .solver import energy_spectrum

    grid = GridSpec(n)
    u0 = ics.taylor_green(n)
    out = {"workload": f"Taylor-Green N={n}, nu={nu}, fixed dt={dt}, {steps} steps, Tier-1 every step, "
                       f"E(k) at step {steps}", "forms": {}}
    last, spec = {}, {}
    for prec in ("fp64", "fp32bulk"):
        s = Periodic3D(grid, nu, u0, SolverOptions(precision=prec, dt_mode="fixed", dt_fixed=dt, device=device))
        s.run(3, every=1)                     # warm-up (kernel set-up)
        s.restore_state(u0, 0.0, 0, dt)
        t0 = time.perf_counter()
        recs = s.run(steps, every=1)
        _, spec[prec] = energy_spectrum(s)
        wall = time.perf_counter() - t0
        s.restore_state(u0, 0.0, 0, dt)
        rate = 1000.0 * steps / s.step_timed(steps)
        last[prec] = recs[-1]
        s.close()
        out["forms"][prec] = {"steps_per_s_with_diagnostics": steps / wall, "steps_per_s": rate,
                              "energy": last[prec].energy, "enstrophy": last[prec].enstrophy,
                              "max_vorticity": last[prec].max_vorticity,
                              "spectrum_sum": float(np.sum(spec[prec]))}
    a, b = spec["fp64"], spec["fp32bulk"]
    keep = a > 1e-12 * a.max()
    out["fp32bulk_rel_error"] = {k: abs(getattr(last["fp32bulk"], k) - getattr(last["fp64"], k)) /
                                 abs(getattr(last["fp64"], k)) for k in ("energy", "enstrophy", "max_vorticity")}
    out["fp32bulk_rel_error"]["spectrum_max_rel_shell"] = float(np.max(np.abs(b - a)[keep] / a[keep]))
    return out


def isotropic(n: int = 256, nu: float = 1e-3, t_end: float = 2.0, spectrum_every: int = 10,
              device: int = 0) -> dict:
    from .solver import energy_spectrum

    grid = GridSpec(n)
    u0 = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=42)
    out = {"workload": f"random isotropic von Karman kp=4 E=0.5 seed 42, N={n}, nu={nu}, adaptive CFL 0.5, "
                       f"to t={t_end}, Tier-1 every step, E(k) every {spectrum_every} steps", "forms": {}}
    series, spectra = {}, {}
    for prec in ("fp64", "fp32bulk"):
        s = Periodic3D(grid, nu, u0, SolverOptions(precision=prec, device=device))
        recs, specs = [], []
        t0 = time.perf_counter()
        while s.time() < t_end:
            recs.extend(s.run(1, every=1))
            if s.step_count() % spectrum_every == 0:
                specs.append(energy_spectrum(s)[1])
        wall = time.perf_counter() - t0
        series[prec], spectra[prec] = recs, specs
        out["forms"][prec] = {"steps": len(recs), "t_last": recs[-1].time, "wall_s": wall,
                              "steps_per_s_with_diagnostics": len(recs) / wall,
                              "energy_t_end": interp_at(recs, t_end, "energy"),
                              "enstrophy_t_end": interp_at(recs, t_end, "enstrophy"),
                              "max_vorticity_t_end": interp_at(recs, t_end, "max_vorticity")}
        s.close()
    f64, f32 = out["forms"]["fp64"], out["forms"]["fp32bulk"]
    out["rel_error_at_t_end"] = {k: abs(f32[k + "_t_end"] - f64[k + "_t_end"]) / abs(f64[k + "_t_end"])
                                 for k in ("energy", "enstrophy", "max_vorticity")}
    k = min(len(spectra["fp64"]), len(spectra["fp32bulk"]))
    if k:
        a, b = spectra["fp64"][k - 1], spectra["fp32bulk"][k - 1]
        keep = a > 1e-12 * a.max()
        out["spectrum_max_rel_shell_last_common"] = float(np.max(np.abs(b - a)[keep] / a[keep]))
    return out


def _grad_rel(g, g_ref, n: int) -> float:
    d = [a - b for a, b in zip(g, g_ref)]
    return math.sqrt(l2_inner(d, d, n) / l2_inner(g_ref, g_ref, n))


def ascent(n: int = 256, nu: float = 2e-3, dt: float = 1e-3, nsteps: int = 1000, nsnap: int = 20,
           iters: int = 10, device: int = 0, schedule: str = "two-level") -> dict:
    grid = GridSpec(n)
    u0 = ics.project_control(ics.von_karman_isotropic(n, kp=3.0, energy=0.5, seed=42), n)
    r = math.sqrt(l2_inner(u0, u0, n))
    u0 = [c / r for c in u0]          # on the sphere <u, u> = 1 (E = 0.5)
    out = {"workload": f"random isotropic kp=3 E=0.5, N={n}, nu={nu}, fixed dt={dt}, {nsteps} steps, "
                       f"{nsnap} saved states, {schedule} schedule", "forms": {}}
    grads = {}
    for prec in ("fp64", "fp32bulk"):
        s = Periodic3D(grid, nu, u0, SolverOptions(precision=prec, dt_mode="fixed", dt_fixed=dt, device=device))
        s.step(2)
        s.restore_state(u0, 0.0, 0, dt)
        s.event_mark(0)
        s.step(nsteps)
        s.event_mark(1)
        s.restore_state(u0, 0.0, 0, dt)
        s.event_mark(2)
        # the FP64 gradient is the reference for the FP32-bulk one; both
        # schedules give the same gradient, the two-level one in less time
        sched = schedule if prec == "fp32bulk" else "two-level"
        J = s.adjoint_forward(nsteps, nsnap, schedule=sched)
        s.event_mark(3)
        grads[prec] = s.adjoint_backward()
        s.event_mark(4)
        fwd, af, ab = s.event_elapsed(0, 1), s.event_elapsed(2, 3), s.event_elapsed(3, 4)
        out["forms"][prec] = {"schedule": sched, "J": J, "forward_ms": fwd, "adjoint_forward_ms": af, "adjoint_backward_ms": ab,
                              "total_over_forward": (af + ab) / fwd,
                              "gradient_norm": math.sqrt(l2_inner(grads[prec], grads[prec], n))}
        s.close()
    out["fp32bulk_vs_fp64_gradient_rel_l2"] = _grad_rel(grads["fp32bulk"], grads["fp64"], n)
    out["fp32bulk_vs_fp64_J_rel"] = abs(out["forms"]["fp32bulk"]["J"] - out["forms"]["fp64"]["J"]) / abs(
        out["forms"]["fp64"]["J"])
    del grads
    t0 = time.perf_counter()
    res = optimize.enstrophy_ascent(grid, nu, dt, u0, nsteps, iters=iters, nsnap=nsnap, precision="fp32bulk",
                                    schedule=schedule)
    out["ascent"] = {"iterations": iters, "J": res.J, "grad_norm": res.grad_norm,
                     "energy_final": 0.5 * l2_inner(res.u, res.u, n), "wall_s": time.perf_counter() - t0}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("workload", choices=["tg", "isotropic", "tubes", "ascent"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--t-end", type=float, default=None)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--schedule", choices=["two-level", "binomial"], default="two-level",
                    help="checkpoint schedule of the ascent workload")
    a = ap.parse_args(argv)
    if a.workload == "tg":
        r = tg(n=a.n or 64, device=a.device)
    elif a.workload == "isotropic":
        r = isotropic(n=a.n or 256, t_end=a.t_end or 2.0, device=a.device)
    elif a.workload == "tubes":
        r = tubes(n=a.n or 512, t_end=a.t_end or 5.0, device=a.device)
    else:
        r = ascent(n=a.n or 256, nsteps=a.steps, iters=a.iters, device=a.device, schedule=a.schedule)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
