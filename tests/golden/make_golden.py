"""Generates the golden fixtures under tests/golden/ with the numpy oracle.

    python tests/golden/make_golden.py

Fixtures (compressed .npz, inputs and outputs in the reference layout):
  tg64_fixed.npz   Taylor-Green N=64, nu=6.25e-4, fixed dt=1e-3: Tier-1 after
                   every step for 100 steps, E(k) at step 100, and norms of
                   u_hat after one step.
  rand16_cfl.npz   seeded Hermitian random state N=16: compute_nonlinear of it,
                   and the state, dt and time after 1 and 5 adaptive-CFL steps.
  rand8_fixed.npz  N=8 random state, RK4 and Cox-Matthews ETD after 2 fixed steps.
  fft_small.npz    r2c/c2r of seeded real arrays on (8,8,8), (12,16,24).
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import vk_oracle as vo  # noqa: E402

TIER1_KEYS = ["time", "step", "dt", "energy", "enstrophy", "helicity", "superhelicity", "max_vorticity",
              "energy_dissipation_rate", "helicity_dissipation_rate", "cfl_number"]


def tier1_row(s):
    d = s.tier1()
    return [float(d[k]) for k in TIER1_KEYS]


def make_tg64():
    n, nu, dt = 64, 6.25e-4, 1e-3
    g = vo.Grid(n)
    s = vo.Periodic3D(g, nu, vo.taylor_green(g), dt_mode="fixed", dt_fixed=dt)
    rows = [tier1_row(s)]
    norms1 = None
    for k in range(100):
        s.step()
        if k == 0:
            norms1 = np.array([np.sqrt(np.sum(np.abs(c) ** 2)) for c in s.u_hat])
            sample1 = np.stack([c[:4, :4, :4] for c in s.u_hat])
        rows.append(tier1_row(s))
    shells, spec = vo.energy_spectrum(s.u_hat, s.ops)
    np.savez_compressed(os.path.join(HERE, "tg64_fixed.npz"), tier1=np.array(rows), keys=np.array(TIER1_KEYS),
                        shells=shells, spectrum=spec, norms_step1=norms1, sample_step1=sample1,
                        n=n, nu=nu, dt=dt)


def make_rand16():
    n, nu = 16, 0.02
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 3, amp=float(n) ** 3 / 40.0))
    nl = vo.compute_nonlinear(vo.SpectralOps(g), u0)
    s = vo.Periodic3D(g, nu, u0)
    dt0 = s.dt
    s.step()
    u1, dt1, t1 = [c.copy() for c in s.u_hat], s.dt, s.time
    for _ in range(4):
        s.step()
    np.savez_compressed(os.path.join(HERE, "rand16_cfl.npz"), u0=np.stack(u0), nl0=np.stack(nl), dt0=dt0,
                        u1=np.stack(u1), dt1=dt1, t1=t1, u5=np.stack(s.u_hat), dt5=s.dt, t5=s.time,
                        tier1_5=np.array(tier1_row(s)), n=n, nu=nu)


def make_rand8():
    n, nu, dt = 8, 0.05, 0.01
    g = vo.Grid(n)
    u0 = vo.hermitian_clean(g, vo.random_field(g, 11, amp=20.0))
    out = {"u0": np.stack(u0), "n": n, "nu": nu, "dt": dt}
    for name, kw in (("rk4", dict(integrator="rk4")), ("cm", dict(etd_variant="cox-matthews")),
                     ("ref", dict())):
        s = vo.Periodic3D(g, nu, u0, dt_mode="fixed", dt_fixed=dt, **kw)
        s.step()
        s.step()
        out["u2_" + name] = np.stack(s.u_hat)
    np.savez_compressed(os.path.join(HERE, "rand8_fixed.npz"), **out)


def make_fft():
    rng = np.random.default_rng(123)
    out = {}
    for i, shp in enumerate([(8, 8, 8), (12, 16, 24)]):
        x = rng.standard_normal(shp)
        xh = vo.r2c_3d(x)
        yh = xh + 0.25j * rng.standard_normal(xh.shape)  # non-Hermitian DC/Nyquist planes too
        out[f"x{i}"] = x
        out[f"xh{i}"] = xh
        out[f"yh{i}"] = yh
        out[f"y{i}"] = vo.c2r_3d(yh, shp)
    np.savez_compressed(os.path.join(HERE, "fft_small.npz"), **out)


if __name__ == "__main__":
    make_fft()
    make_rand8()
    make_rand16()
    make_tg64()
    print("fixtures written to", HERE)
