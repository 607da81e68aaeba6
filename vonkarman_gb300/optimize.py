"""Gradient checks and enstrophy-growth search over initial conditions with
the discrete adjoint (vk_adjoint_forward / vk_adjoint_backward).

The control is the initial state in the space of real, divergence-free,
Nyquist-free fields; inner products are the L2 inner product of the physical
fields (``l2_inner``), so the "unit-energy sphere" is <u, u> = 1, i.e.
E = 0.5.  The objective is the final enstrophy in the reference's convention
(<|omega|^2>, vonkarman-periodic/src/solver.rs:436-465).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import ics
from .solver import GridSpec, Periodic3D, SolverOptions, l2_inner


def _axpy(a, x, y):
    return [a * xi + yi for xi, yi in zip(x, y)]


def gradient(solver: Periodic3D, u0, nsteps: int, nsnap: int = 20, schedule: str = "two-level"):
    """J(u0) and dJ/du0 with the solver's configuration (fixed dt); schedule
    is the checkpoint schedule of the adjoint ("two-level" or "binomial")."""
    solver.restore_state(u0, 0.0, 0, solver.options.dt_fixed)
    J = solver.adjoint_forward(nsteps, nsnap, schedule=schedule)
    return J, solver.adjoint_backward()


def fd_check(grid: GridSpec, nu: float, dt: float, u0, nsteps: int, seeds, eps: float = 1e-6,
             precision: str = "fp64", nsnap: int = 20, kp: float = 8.0):
    """Central finite differences of J along seeded solenoidal directions
    against the adjoint directional derivative <v, grad J>."""
    opts = SolverOptions(precision=precision, dt_mode="fixed", dt_fixed=dt)
    s = Periodic3D(grid, nu, u0, opts)
    J, g = gradient(s, u0, nsteps, nsnap)
    out = []
    for seed in seeds:
        v = ics.solenoidal_direction(grid.n, seed=seed, kp=kp, l=grid.l)
        s.restore_state(_axpy(eps, v, u0), 0.0, 0, dt)
        jp = s.adjoint_forward(nsteps, nsnap)
        s.restore_state(_axpy(-eps, v, u0), 0.0, 0, dt)
        jm = s.adjoint_forward(nsteps, nsnap)
        fd = (jp - jm) / (2.0 * eps)
        ad = l2_inner(v, g, grid.n)
        out.append({"seed": seed, "fd": fd, "adjoint": ad, "rel": abs(fd - ad) / max(abs(fd), 1e-300)})
    s.close()
    return J, out


@dataclass
class AscentResult:
    u: list
    J: list = field(default_factory=list)
    grad_norm: list = field(default_factory=list)


def enstrophy_ascent(grid: GridSpec, nu: float, dt: float, u0, nsteps: int, iters: int = 10, nsnap: int = 20,
                     precision: str = "fp32bulk", step: float = 0.2, schedule: str = "two-level") -> AscentResult:
    """Projected-gradient ascent of the final enstrophy on the sphere
    <u, u> = <u0, u0>: the gradient is projected on the tangent space, the
    step length is ``step`` times the radius, and the iterate is pulled back
    to the sphere."""
    n = grid.n
    u = ics.project_control(u0, n, grid.l)
    r2 = l2_inner(u0, u0, n)
    u = [c * math.sqrt(r2 / l2_inner(u, u, n)) for c in u]
    s = Periodic3D(grid, nu, u, SolverOptions(precision=precision, dt_mode="fixed", dt_fixed=dt))
    res = AscentResult(u=u)
    for _ in range(iters):
        J, g = gradient(s, u, nsteps, nsnap, schedule)
        gt = _axpy(-l2_inner(g, u, n) / r2, u, g)
        gn = math.sqrt(max(l2_inner(gt, gt, n), 0.0))
        res.J.append(J)
        res.grad_norm.append(gn)
        if gn == 0.0:
            break
        un = _axpy(step * math.sqrt(r2) / gn, gt, u)
        u = [c * math.sqrt(r2 / l2_inner(un, un, n)) for c in un]
    s.restore_state(u, 0.0, 0, dt)
    res.J.append(s.adjoint_forward(nsteps, nsnap, schedule=schedule))
    res.u = u
    s.close()
    return res
