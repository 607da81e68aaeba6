"""Discrete adjoint of the restated ETD-RK4 step (numpy, FP64).

TEST INFRASTRUCTURE ONLY.  The reference has no adjoint; this is an
independent, hand-derived transpose of the oracle's forward map
(``vk_oracle.Periodic3D`` with the reference ETD variant and a fixed dt), used
to check the GPU adjoint and, itself, checked against central finite
differences (``tests/test_adjoint_oracle.py``).

Conventions.  States are the stored R2C arrays (n, n, n/2+1) x 3.  Adjoints
are taken in the raw Euclidean inner product  <a, b> = Re sum conj(a) b  over
the stored entries.  With it:
  * r2c  F:  F^T Y = C2R_unnorm(Y / w)         (w = R2C weight of the grid)
  * c2r  G = C2R_unnorm / n^3:  G^T y = (w / n^3) F y
  * zero-pad and truncation are mutual transposes; curl (i k x) and the
    Leray projector are self-adjoint per mode; ETD coefficients are real.
The objective is the final enstrophy  J = sum w |curl u|^2 / N^6
(solver.rs:436-465), whose raw gradient is (2/N^6) w curl curl u.
The gradient is finally expressed in the weighted inner product
<a, b>_w = Re sum w conj(a) b / N^6 (the L2 inner product of the physical
fields), Leray-projected and made Hermitian on the kz = 0, N/2 planes.
"""

from __future__ import annotations

import numpy as np

from . import vk_oracle as vo


def _w(n: int, h: int, padded_interior_nyquist: bool = False):
    """R2C weight over kz in [0, h): 1 at kz = 0 and at the grid's own Nyquist."""
    w = np.full(h, 2.0)
    w[0] = 1.0
    if not padded_interior_nyquist and h - 1 == n // 2:
        w[-1] = 1.0
    return w[None, None, :]


def cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def nonlinear_adjoint(ops: vo.SpectralOps, x, nbar):
    """y = N'(x)^T nbar for N(x) = P T S_out F_M cross(G_M S_in Pad x, G_M S_in Pad curl x)."""
    g = ops.grid
    n, m = g.n, g.m
    scale = float(m ** 3) / float(n ** 3)
    shp = (m, m, m)
    hm = m // 2 + 1
    wm_full = _w(m, hm)                       # padded grid weights over all padded kz
    om = ops.curl(x)
    up = [vo.c2r_3d(vo.zero_pad_spectral(c, n, m) * scale, shp) for c in x]
    wp = [vo.c2r_3d(vo.zero_pad_spectral(c, n, m) * scale, shp) for c in om]
    pn = ops.leray_project(nbar)
    # c_bar = F_M^T Pad(S_out P nbar) = C2R_unnorm(Pad(P nbar) / scale / w_M)
    cbar = [vo.c2r_3d(vo.zero_pad_spectral(c, n, m) / scale / wm_full, shp) * float(m ** 3) for c in pn]
    abar = cross(wp, cbar)   # cotangent of u_phys:  omega x c_bar
    obar = cross(cbar, up)   # cotangent of omega_phys: c_bar x u
    wm_kept = wm_full[:, :, : g.h]
    nt = float(n ** 3)
    ya = [vo.truncate_spectral(vo.r2c_3d(c), n, m) * wm_kept / nt for c in abar]
    yo = [vo.truncate_spectral(vo.r2c_3d(c), n, m) * wm_kept / nt for c in obar]
    co = ops.curl(yo)
    return [ya[c] + co[c] for c in range(3)]


def step_adjoint(s: vo.Periodic3D, u, ubar):
    """Adjoint of one reference-variant ETD-RK4 step taken from state u with
    s's (fixed) dt and ETD table: returns dJ/du given dJ/du_next = ubar."""
    ec, dt, ops = s.etd, s.dt, s.ops
    n1 = vo.compute_nonlinear(ops, u)
    a = [ec.exp_half * u[c] + dt * ec.a21 * n1[c] for c in range(3)]
    n2 = vo.compute_nonlinear(ops, a)
    b = [ec.exp_half * u[c] + dt * ec.a31 * n2[c] for c in range(3)]
    n3 = vo.compute_nonlinear(ops, b)
    cc = [ec.exp_full * u[c] + dt * ec.a41 * (2.0 * n3[c] - n1[c]) for c in range(3)]
    # reverse
    n4b = [dt * ec.b4 * ubar[c] for c in range(3)]
    cb = nonlinear_adjoint(ops, cc, n4b)
    acc = [ec.exp_full * ubar[c] + ec.exp_full * cb[c] for c in range(3)]
    n3b = [dt * ec.b23 * ubar[c] + 2.0 * dt * ec.a41 * cb[c] for c in range(3)]
    n1b = [dt * ec.b1 * ubar[c] - dt * ec.a41 * cb[c] for c in range(3)]
    bb = nonlinear_adjoint(ops, b, n3b)
    acc = [acc[c] + ec.exp_half * bb[c] for c in range(3)]
    n2b = [dt * ec.b23 * ubar[c] + dt * ec.a31 * bb[c] for c in range(3)]
    ab = nonlinear_adjoint(ops, a, n2b)
    acc = [acc[c] + ec.exp_half * ab[c] for c in range(3)]
    n1b = [n1b[c] + dt * ec.a21 * ab[c] for c in range(3)]
    ub = nonlinear_adjoint(ops, u, n1b)
    return [acc[c] + ub[c] for c in range(3)]


def enstrophy_grad_raw(ops: vo.SpectralOps, u):
    g = ops.grid
    nt2 = float(g.n ** 3) ** 2
    w = _w(g.n, g.h)
    cc = ops.curl(ops.curl(u))
    return [2.0 * w * c / nt2 for c in cc]


def hermitian_symmetrize(g: vo.Grid, a):
    """Average each kz in {0, n/2} plane with its (kx, ky) -> (-kx, -ky)
    conjugate, so the field is the one a real physical field would have."""
    n = g.n
    idx = (-np.arange(n)) % n
    out = []
    for c in a:
        c = c.copy()
        for kz in (0, n // 2):
            p = c[:, :, kz]
            c[:, :, kz] = 0.5 * (p + np.conj(p[np.ix_(idx, idx)]))
        out.append(c)
    return out


def zero_nyquist(g: vo.Grid, a):
    """Zero the entries with ix = n/2, iy = n/2 or iz = n/2.  With the
    reference's convention kx[n/2] = -n/2 (spectral_ops.rs:58-61) a field can
    be both Hermitian and divergence-free there only if they vanish."""
    n = g.n
    out = []
    for c in a:
        c = c.copy()
        c[n // 2, :, :] = 0.0
        c[:, n // 2, :] = 0.0
        c[:, :, n // 2] = 0.0
        out.append(c)
    return out


def project_control(ops: vo.SpectralOps, a):
    """Orthogonal projection (weighted inner product) onto the control space:
    real (Hermitian), divergence-free fields with zero Nyquist entries."""
    g = ops.grid
    return hermitian_symmetrize(g, ops.leray_project(zero_nyquist(g, a)))


def to_weighted(ops: vo.SpectralOps, graw):
    """Raw-Euclidean gradient -> gradient in <a,b>_w, projected onto the
    control space."""
    g = ops.grid
    nt2 = float(g.n ** 3) ** 2
    w = _w(g.n, g.h)
    return project_control(ops, [c * nt2 / w for c in graw])


def weighted_inner(g: vo.Grid, a, b) -> float:
    w = _w(g.n, g.h)
    nt2 = float(g.n ** 3) ** 2
    return float(sum((w * (np.conj(x) * y).real).sum() for x, y in zip(a, b))) / nt2


def forward_J(grid: vo.Grid, nu: float, dt: float, u0, nsteps: int):
    s = vo.Periodic3D(grid, nu, u0, dt_mode="fixed", dt_fixed=dt)
    for _ in range(nsteps):
        s.step()
    return s.enstrophy(), s


def gradient(grid: vo.Grid, nu: float, dt: float, u0, nsteps: int):
    """J and dJ/du0 (weighted inner product) by storing every state."""
    s = vo.Periodic3D(grid, nu, u0, dt_mode="fixed", dt_fixed=dt)
    states = [[c.copy() for c in s.u_hat]]
    for _ in range(nsteps):
        s.step()
        states.append([c.copy() for c in s.u_hat])
    J = s.enstrophy()
    ubar = enstrophy_grad_raw(s.ops, s.u_hat)
    for k in range(nsteps - 1, -1, -1):
        ubar = step_adjoint(s, states[k], ubar)
    return J, to_weighted(s.ops, ubar), ubar
