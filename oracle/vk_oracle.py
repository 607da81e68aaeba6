"""FP64 numpy restatement of vonkarman's periodic pseudospectral step.

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the CUDA library is
checked against.  Only the test suite, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it; the
product path (``vonkarman_gb300``) never does.

Every function below restates one piece of the reference (alejandro-soto-franco/
vonkarman, Rust) and cites the file:line it follows.  The reference itself
cannot be compiled in this environment (no Rust toolchain), and its FFT lives
in the third-party crate ``ndrustfft`` 0.5 (-> ``rustfft``/``realfft``; the
patch versions are unpinned because the reference ships no ``Cargo.lock``).
That crate's published semantics are restated with numpy's pocketfft:

* ``r2c_3d`` = unnormalised forward transform: z real-to-complex, then y and x
  complex-to-complex (``vonkarman-fft/src/ndrustfft_backend.rs:33-44``).
* ``c2r_3d`` = inverse with the 1/(nx*ny*nz) normalisation folded in: x and y
  inverse complex-to-complex, then z complex-to-real; the imaginary parts of
  the z=0 and z=nz/2 planes are ignored (``ndrustfft_backend.rs:46-57``).

Parity pin: the restatement is checked against every known-answer and
invariant test the reference holds for this path (``tests/test_oracle_kats.py``
lists them with their reference file:line).  The reference ships no stored
step outputs, so exact step values are anchored on this restatement.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * math.pi

# ---------------------------------------------------------------------------
# Grid and wavenumbers  (vonkarman-core/src/field.rs, spectral_ops.rs)
# ---------------------------------------------------------------------------


@dataclass(frozen=True)
class Grid:
    """Cubic periodic grid, ``GridSpec::cubic`` (field.rs:18-27)."""

    n: int
    l: float = TWO_PI

    @property
    def h(self) -> int:  # spectral_shape() z extent, field.rs:48-50
        return self.n // 2 + 1

    @property
    def m(self) -> int:  # padded_3half(), field.rs:53-62
        return 3 * self.n // 2

    @property
    def dx(self) -> float:  # field.rs:30-32
        return self.l / self.n

    @property
    def spectral_shape(self):
        return (self.n, self.n, self.h)


def rfftfreq_full(n: int, l: float) -> np.ndarray:
    """spectral_ops.rs:51-63 -- index n/2 maps to -n/2."""
    scale = 2.0 * math.pi / l
    k = np.empty(n, dtype=np.float64)
    k[: n // 2] = np.arange(n // 2, dtype=np.float64) * scale
    k[n // 2 :] = (np.arange(n // 2, n, dtype=np.float64) - float(n)) * scale
    return k


def rfftfreq_half(n: int, l: float) -> np.ndarray:
    """spectral_ops.rs:66-74."""
    scale = 2.0 * math.pi / l
    return np.arange(n // 2 + 1, dtype=np.float64) * scale


class SpectralOps:
    """``SpectralOps<f64>`` (spectral_ops.rs:10-48)."""

    def __init__(self, grid: Grid):
        self.grid = grid
        self.kx = rfftfreq_full(grid.n, grid.l)
        self.ky = rfftfreq_full(grid.n, grid.l)
        self.kz = rfftfreq_half(grid.n, grid.l)
        KX = self.kx[:, None, None]
        KY = self.ky[None, :, None]
        KZ = self.kz[None, None, :]
        # spectral_ops.rs:36  kx*kx + ky*ky + kz*kz (left to right)
        self.k_mag_sq = (KX * KX + KY * KY) + KZ * KZ
        self.KX, self.KY, self.KZ = KX, KY, KZ

    def curl(self, u):
        """omega_hat = i k x u_hat (spectral_ops.rs:81-108)."""
        KX, KY, KZ = self.KX, self.KY, self.KZ
        ux, uy, uz = u
        ox = (-(KY * uz.imag - KZ * uy.imag)) + 1j * (KY * uz.real - KZ * uy.real)
        oy = (-(KZ * ux.imag - KX * uz.imag)) + 1j * (KZ * ux.real - KX * uz.real)
        oz = (-(KX * uy.imag - KY * ux.imag)) + 1j * (KX * uy.real - KY * ux.real)
        return [ox, oy, oz]

    def leray_project(self, u):
        """u -= k (k.u)/|k|^2, k=0 untouched (spectral_ops.rs:114-151).  Returns new list."""
        KX, KY, KZ = self.KX, self.KY, self.KZ
        k2 = self.k_mag_sq
        skip = k2 < 1e-30
        with np.errstate(divide="ignore", invalid="ignore"):
            inv_k2 = np.where(skip, 0.0, 1.0 / np.where(skip, 1.0, k2))
        ux, uy, uz = u
        kdu_re = (KX * ux.real + KY * uy.real) + KZ * uz.real
        kdu_im = (KX * ux.imag + KY * uy.imag) + KZ * uz.imag
        out = []
        for comp, K in ((ux, KX), (uy, KY), (uz, KZ)):
            re = comp.real - K * kdu_re * inv_k2
            im = comp.imag - K * kdu_im * inv_k2
            res = re + 1j * im
            out.append(np.where(skip, comp, res))
        return out

    def apply_viscous(self, u, nu: float):
        """-nu |k|^2 u (spectral_ops.rs:154-175)."""
        factor = -(nu * self.k_mag_sq)
        return [factor * c.real + 1j * (factor * c.imag) for c in u]


# ---------------------------------------------------------------------------
# FFT backend (FftBackend contract, backend.rs:9-25)
# ---------------------------------------------------------------------------


def r2c_3d(x: np.ndarray) -> np.ndarray:
    """Unnormalised forward R2C (ndrustfft_backend.rs:33-44)."""
    return np.fft.rfftn(np.asarray(x, dtype=np.float64))


def c2r_3d(xh: np.ndarray, shape) -> np.ndarray:
    """Inverse C2R including 1/N^3 (ndrustfft_backend.rs:46-57)."""
    return np.fft.irfftn(np.asarray(xh, dtype=np.complex128), s=shape, axes=(0, 1, 2))


# ---------------------------------------------------------------------------
# 3/2 dealiased cross product (vonkarman-fft/src/dealiased.rs)
# ---------------------------------------------------------------------------


def _pad_index(n: int, m: int) -> np.ndarray:
    """dealiased.rs:129-131: ix < n/2 -> ix, else m - (n - ix)."""
    return np.array([i if i < n // 2 else m - (n - i) for i in range(n)], dtype=np.int64)


def zero_pad_spectral(src: np.ndarray, n: int, m: int) -> np.ndarray:
    """(n,n,n/2+1) -> (m,m,m/2+1); z copied 0..n/2 (dealiased.rs:115-138)."""
    dst = np.zeros((m, m, m // 2 + 1), dtype=np.complex128)
    idx = _pad_index(n, m)
    h = src.shape[2]
    dst[np.ix_(idx, idx, np.arange(h))] = src
    return dst


def truncate_spectral(src: np.ndarray, n: int, m: int) -> np.ndarray:
    """(m,m,m/2+1) -> (n,n,n/2+1) (dealiased.rs:141-163)."""
    idx = _pad_index(n, m)
    h = n // 2 + 1
    return src[np.ix_(idx, idx, np.arange(h))].copy()


def dealiased_cross_product(grid: Grid, u_hat, omega_hat):
    """u x omega with 3/2 padding (dealiased.rs:16-110)."""
    n, m = grid.n, grid.m
    scale = float(m * m * m) / float(n * n * n)  # dealiased.rs:43
    shp = (m, m, m)
    up = [c2r_3d(zero_pad_spectral(u_hat[c], n, m) * scale, shp) for c in range(3)]
    op = [c2r_3d(zero_pad_spectral(omega_hat[c], n, m) * scale, shp) for c in range(3)]
    ux, uy, uz = up
    ox, oy, oz = op
    cross = [uy * oz - uz * oy, uz * ox - ux * oz, ux * oy - uy * ox]  # dealiased.rs:70-84
    inv_scale = 1.0 / scale  # dealiased.rs:102
    out = []
    for c in range(3):
        t = truncate_spectral(r2c_3d(cross[c]), n, m)
        out.append(t.real * inv_scale + 1j * (t.imag * inv_scale))
    return out


def compute_nonlinear(ops: SpectralOps, u_hat):
    """N_hat = P[F(u x omega)] (vonkarman-periodic/src/nonlinear.rs:15-39)."""
    omega = ops.curl(u_hat)
    nl = dealiased_cross_product(ops.grid, u_hat, omega)
    return ops.leray_project(nl)


# ---------------------------------------------------------------------------
# ETD coefficients (vonkarman-periodic/src/etd.rs)
# ---------------------------------------------------------------------------

M_CONTOUR = 32  # etd.rs:5


def _contour_points():
    return [2.0 * math.pi * (j + 0.5) / M_CONTOUR for j in range(M_CONTOUR)]


def phi1(z):
    """etd.rs:15-34 (vectorised over z; the j-sum is sequential as in the reference)."""
    z = np.asarray(z, dtype=np.float64)
    s = np.zeros_like(z)
    for th in _contour_points():
        w_re = z + 1.0 * math.cos(th)
        w_im = 1.0 * math.sin(th)
        e = np.exp(w_re)
        ew_re = e * math.cos(w_im)
        ew_im = e * math.sin(w_im)
        num_re = ew_re - 1.0
        num_im = ew_im
        denom = w_re * w_re + w_im * w_im
        s = s + (num_re * w_re + num_im * w_im) / denom
    out = s / M_CONTOUR
    return np.where(np.abs(z) < 1e-300, 1.0, out)


def phi2(z):
    """etd.rs:37-58."""
    z = np.asarray(z, dtype=np.float64)
    s = np.zeros_like(z)
    for th in _contour_points():
        w_re = z + 1.0 * math.cos(th)
        w_im = 1.0 * math.sin(th)
        e = np.exp(w_re)
        ew_re = e * math.cos(w_im)
        ew_im = e * math.sin(w_im)
        num_re = ew_re - 1.0 - w_re
        num_im = ew_im - w_im
        w2_re = w_re * w_re - w_im * w_im
        w2_im = 2.0 * w_re * w_im
        denom = w2_re * w2_re + w2_im * w2_im
        s = s + (num_re * w2_re + num_im * w2_im) / denom
    out = s / M_CONTOUR
    return np.where(np.abs(z) < 1e-300, 0.5, out)


def phi3(z):
    """etd.rs:61-84."""
    z = np.asarray(z, dtype=np.float64)
    s = np.zeros_like(z)
    for th in _contour_points():
        w_re = z + 1.0 * math.cos(th)
        w_im = 1.0 * math.sin(th)
        e = np.exp(w_re)
        ew_re = e * math.cos(w_im)
        ew_im = e * math.sin(w_im)
        w2_re = w_re * w_re - w_im * w_im
        w2_im = 2.0 * w_re * w_im
        num_re = ew_re - 1.0 - w_re - 0.5 * w2_re
        num_im = ew_im - w_im - 0.5 * w2_im
        w3_re = w_re * w2_re - w_im * w2_im
        w3_im = w_re * w2_im + w_im * w2_re
        denom = w3_re * w3_re + w3_im * w3_im
        s = s + (num_re * w3_re + num_im * w3_im) / denom
    out = s / M_CONTOUR
    return np.where(np.abs(z) < 1e-300, 1.0 / 6.0, out)


@dataclass
class EtdCoeffs:
    """``EtdCoeffs::new`` (etd.rs:113-135); arrays over modes."""

    exp_full: np.ndarray
    exp_half: np.ndarray
    a21: np.ndarray
    a31: np.ndarray
    a41: np.ndarray
    b1: np.ndarray
    b23: np.ndarray
    b4: np.ndarray

    @classmethod
    def new(cls, lambda_dt):
        z = np.asarray(lambda_dt, dtype=np.float64)
        zh = z / 2.0
        p1h = phi1(zh)
        p1f = phi1(z)
        p2f = phi2(z)
        p3f = phi3(z)
        return cls(
            exp_full=np.exp(z),
            exp_half=np.exp(zh),
            a21=p1h,
            a31=p1h,
            a41=p1f,
            b1=p1f - 3.0 * p2f + 4.0 * p3f,
            b23=2.0 * p2f - 4.0 * p3f,
            b4=-p2f + 4.0 * p3f,
        )


# ---------------------------------------------------------------------------
# Solver (vonkarman-periodic/src/solver.rs, rk4.rs)
# ---------------------------------------------------------------------------


def _r2c_weight(grid: Grid) -> np.ndarray:
    """solver.rs:423-427: weight 1 at iz in {0, n/2}, else 2."""
    w = np.full(grid.h, 2.0)
    w[0] = 1.0
    w[grid.n // 2] = 1.0
    return w[None, None, :]


def _cplx(re, im):
    return re + 1j * im


class Periodic3D:
    """Restatement of ``Periodic3D`` (solver.rs:12-618).

    Extra options mirror the GPU library's config (they are not in the
    reference): ``dt_mode`` ("cfl" = the reference, "fixed"), ``cfl_safety``
    (the reference hardcodes 0.5, solver.rs:89), ``etd_variant``
    ("reference" = solver.rs:221-379, "cox-matthews" = textbook stages) and
    ``integrator`` ("etd-rk4" or "rk4" = rk4.rs:16-146).
    """

    def __init__(self, grid: Grid, nu: float, u_hat, *, dt_mode="cfl", dt_fixed=None,
                 cfl_safety=0.5, etd_variant="reference", integrator="etd-rk4",
                 time=0.0, step_count=0, dt=None):
        self.grid = grid
        self.nu = float(nu)
        self.ops = SpectralOps(grid)
        self.u_hat = [np.array(c, dtype=np.complex128, copy=True) for c in u_hat]
        self.dt_mode = dt_mode
        self.dt_fixed = dt_fixed
        self.cfl_safety = cfl_safety
        self.etd_variant = etd_variant
        self.integrator = integrator
        self.time = float(time)
        self.step_count = int(step_count)
        if dt is not None:  # from_checkpoint (solver.rs:127-159)
            self.dt = float(dt)
        elif dt_mode == "fixed":
            self.dt = float(dt_fixed)
        else:  # solver.rs:88-90
            self.dt = self.compute_cfl_dt()
        self._recompute_etd()

    # -- ETD table (solver.rs:161-177) ------------------------------------
    def _recompute_etd(self):
        lam = -self.nu * self.ops.k_mag_sq  # solver.rs:167
        self.etd = EtdCoeffs.new(lam * self.dt)

    # -- CFL (solver.rs:180-218) ------------------------------------------
    def max_speed(self) -> float:
        shp = (self.grid.n,) * 3
        up = [c2r_3d(c, shp) for c in self.u_hat]
        return float(np.sqrt(up[0] ** 2 + up[1] ** 2 + up[2] ** 2).max())

    def compute_cfl_dt(self) -> float:
        u_max = self.max_speed()
        dx = self.grid.dx
        advective = dx / u_max if u_max > 1e-30 else 1.0
        viscous = dx * dx / self.nu if self.nu > 1e-30 else math.inf
        return self.cfl_safety * min(min(advective, viscous), 0.1)

    # -- one step (solver.rs:383-400) -------------------------------------
    def step(self):
        if self.dt_mode == "cfl":
            new_dt = self.compute_cfl_dt()
            if abs(new_dt - self.dt) / max(self.dt, 1e-30) > 0.01:
                self.dt = new_dt
                self._recompute_etd()
        if self.integrator == "rk4":
            self.u_hat = rk4_step(self.u_hat, self.ops, self.nu, self.dt)
        elif self.etd_variant == "reference":
            self._etd_rk4_reference()
        else:
            self._etd_rk4_cox_matthews()
        self.time += self.dt
        self.step_count += 1

    def _etd_rk4_reference(self):
        """solver.rs:221-379, stage formulas kept exactly (incl. dt*phi1(z/2))."""
        ec, dt, u = self.etd, self.dt, self.u_hat
        n1 = compute_nonlinear(self.ops, u)
        temp = [_cplx(ec.exp_half * u[c].real + dt * ec.a21 * n1[c].real,
                      ec.exp_half * u[c].imag + dt * ec.a21 * n1[c].imag) for c in range(3)]
        n2 = compute_nonlinear(self.ops, temp)
        temp = [_cplx(ec.exp_half * u[c].real + dt * ec.a31 * n2[c].real,
                      ec.exp_half * u[c].imag + dt * ec.a31 * n2[c].imag) for c in range(3)]
        n3 = compute_nonlinear(self.ops, temp)
        temp = []
        for c in range(3):
            dn_re = 2.0 * n3[c].real - n1[c].real
            dn_im = 2.0 * n3[c].imag - n1[c].imag
            temp.append(_cplx(ec.exp_full * u[c].real + dt * ec.a41 * dn_re,
                              ec.exp_full * u[c].imag + dt * ec.a41 * dn_im))
        n4 = compute_nonlinear(self.ops, temp)
        new = []
        for c in range(3):
            rhs_re = ec.b1 * n1[c].real + ec.b23 * (n2[c].real + n3[c].real) + ec.b4 * n4[c].real
            rhs_im = ec.b1 * n1[c].imag + ec.b23 * (n2[c].imag + n3[c].imag) + ec.b4 * n4[c].imag
            new.append(_cplx(ec.exp_full * u[c].real + dt * rhs_re,
                             ec.exp_full * u[c].imag + dt * rhs_im))
        self.u_hat = new

    def _etd_rk4_cox_matthews(self):
        """Textbook ETD-RK4 (Cox & Matthews 2002; Kassam & Trefethen 2005 eq. 26):
        a = E2 u + (h/2)phi1(z/2) N(u);  b = E2 u + (h/2)phi1(z/2) N(a);
        c = E2 a + (h/2)phi1(z/2) (2N(b) - N(u));  final as in the reference."""
        ec, dt, u = self.etd, self.dt, self.u_hat
        q = 0.5 * dt * ec.a21
        n1 = compute_nonlinear(self.ops, u)
        a = [ec.exp_half * u[c] + q * n1[c] for c in range(3)]
        n2 = compute_nonlinear(self.ops, a)
        b = [ec.exp_half * u[c] + q * n2[c] for c in range(3)]
        n3 = compute_nonlinear(self.ops, b)
        cc = [ec.exp_half * a[c] + q * (2.0 * n3[c] - n1[c]) for c in range(3)]
        n4 = compute_nonlinear(self.ops, cc)
        self.u_hat = [ec.exp_full * u[c] + dt * (ec.b1 * n1[c] + ec.b23 * (n2[c] + n3[c]) + ec.b4 * n4[c])
                      for c in range(3)]

    # -- Tier-1 diagnostics (solver.rs:412-567) ----------------------------
    def _wsum(self, vals) -> float:
        return float((_r2c_weight(self.grid) * vals).sum())

    def _ntot2(self) -> float:
        nt = float(self.grid.n ** 3)
        return nt * nt

    def energy(self) -> float:
        s = sum(self._wsum(c.real ** 2 + c.imag ** 2) for c in self.u_hat)
        return 0.5 * s / self._ntot2()

    def enstrophy(self) -> float:
        om = self.ops.curl(self.u_hat)
        return sum(self._wsum(c.real ** 2 + c.imag ** 2) for c in om) / self._ntot2()

    def helicity(self) -> float:
        om = self.ops.curl(self.u_hat)
        return sum(self._wsum(u.real * o.real + u.imag * o.imag)
                   for u, o in zip(self.u_hat, om)) / self._ntot2()

    def superhelicity(self) -> float:
        om = self.ops.curl(self.u_hat)
        co = self.ops.curl(om)
        return sum(self._wsum(o.real * c.real + o.imag * c.imag)
                   for o, c in zip(om, co)) / self._ntot2()

    def max_vorticity(self) -> float:
        shp = (self.grid.n,) * 3
        om = [c2r_3d(c, shp) for c in self.ops.curl(self.u_hat)]
        return float(np.sqrt(om[0] ** 2 + om[1] ** 2 + om[2] ** 2).max())

    def tier1(self) -> dict:
        """ScalarDiagnostics::from_domain (vonkarman-diag/src/scalar.rs:22-54)."""
        ens = self.enstrophy()
        sh = self.superhelicity()
        mw = self.max_vorticity()
        return dict(time=self.time, step=self.step_count, dt=self.dt,
                    energy=self.energy(), enstrophy=ens, helicity=self.helicity(),
                    superhelicity=sh, max_vorticity=mw,
                    energy_dissipation_rate=-2.0 * self.nu * ens,
                    helicity_dissipation_rate=-2.0 * self.nu * sh,
                    cfl_number=mw * self.dt / self.grid.dx)


def tier1_of_state(grid: Grid, nu: float, u_hat, time: float, step_count: int, dt: float) -> dict:
    """``ScalarDiagnostics::from_domain`` (vonkarman-diag/src/scalar.rs:22-54) of a
    given state with its time, step count and dt, without building the
    per-mode ETD table of ``Periodic3D.__init__`` (large grids)."""
    p = Periodic3D.__new__(Periodic3D)
    p.grid = grid
    p.nu = float(nu)
    p.ops = SpectralOps(grid)
    p.u_hat = [np.asarray(c, dtype=np.complex128) for c in u_hat]
    p.time, p.step_count, p.dt = float(time), int(step_count), float(dt)
    return p.tier1()


def rk4_step(u_hat, ops: SpectralOps, nu: float, dt: float):
    """Classical RK4 on L + N (rk4.rs:16-146)."""
    k2 = ops.k_mag_sq

    def rhs(state):
        r = compute_nonlinear(ops, state)
        visc = -nu * k2
        return [_cplx(r[c].real + visc * state[c].real, r[c].imag + visc * state[c].imag)
                for c in range(3)]

    k1 = rhs(u_hat)
    temp = [_cplx(u_hat[c].real + 0.5 * dt * k1[c].real, u_hat[c].imag + 0.5 * dt * k1[c].imag)
            for c in range(3)]
    kk2 = rhs(temp)
    temp = [_cplx(u_hat[c].real + 0.5 * dt * kk2[c].real, u_hat[c].imag + 0.5 * dt * kk2[c].imag)
            for c in range(3)]
    kk3 = rhs(temp)
    temp = [_cplx(u_hat[c].real + dt * kk3[c].real, u_hat[c].imag + dt * kk3[c].imag)
            for c in range(3)]
    kk4 = rhs(temp)
    sixth = dt / 6.0
    out = []
    for c in range(3):
        re = u_hat[c].real + sixth * (k1[c].real + 2.0 * kk2[c].real + 2.0 * kk3[c].real + kk4[c].real)
        im = u_hat[c].imag + sixth * (k1[c].imag + 2.0 * kk2[c].imag + 2.0 * kk3[c].imag + kk4[c].imag)
        out.append(_cplx(re, im))
    return out


# ---------------------------------------------------------------------------
# Tier-2 spectrum (vonkarman-diag/src/spectrum.rs)
# ---------------------------------------------------------------------------


def n_shells(grid: Grid) -> int:
    """spectrum.rs:22-26."""
    kmax = (grid.n // 2)
    k_max = math.sqrt(float(kmax * kmax) * 3.0)
    return int(math.ceil(k_max)) + 1


def energy_spectrum(u_hat, ops: SpectralOps):
    """Shell E(k), shell = round(|k|) (spectrum.rs:13-60).  Rust's f64::round
    rounds half away from zero; |k| >= 0 so floor(x + 0.5) matches."""
    grid = ops.grid
    ns = n_shells(grid)
    kmag = np.sqrt(ops.k_mag_sq)
    shell = np.floor(kmag + 0.5).astype(np.int64)
    mag2 = sum(c.real ** 2 + c.imag ** 2 for c in u_hat)
    ntot = float(grid.n ** 3)
    w = np.broadcast_to(_r2c_weight(grid), mag2.shape)
    contrib = 0.5 * w * mag2 / (ntot * ntot)
    keep = shell < ns
    spec = np.bincount(shell[keep].ravel(), weights=contrib[keep].ravel(), minlength=ns)[:ns]
    return np.arange(ns, dtype=np.float64), spec


def compensated_spectrum(shells, spec):
    """spectrum.rs:66-72."""
    shells = np.asarray(shells)
    return np.where(shells > 0.0, np.power(shells, 5.0 / 3.0) * spec, 0.0)


def dissipation_spectrum(shells, spec, nu):
    """spectrum.rs:77-83."""
    shells = np.asarray(shells)
    return 2.0 * nu * shells * shells * spec


# ---------------------------------------------------------------------------
# Initial conditions
# ---------------------------------------------------------------------------


def _coords(grid: Grid):
    x = np.arange(grid.n, dtype=np.float64) * grid.l / grid.n
    return x


def taylor_green(grid: Grid):
    """ic/taylor_green.rs:10-38 -> spectral via r2c (solver.rs:74-76)."""
    x = _coords(grid)
    X, Y, Z = x[:, None, None], x[None, :, None], x[None, None, :]
    ux = np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -(np.cos(X) * np.sin(Y) * np.cos(Z))
    uz = np.zeros((grid.n,) * 3)
    ux = np.broadcast_to(ux, (grid.n,) * 3)
    uy = np.broadcast_to(uy, (grid.n,) * 3)
    return [r2c_3d(ux), r2c_3d(uy), r2c_3d(uz)]


def abc_flow(grid: Grid, a=1.0, b=1.0, c=1.0):
    """ic/abc.rs:14-42."""
    x = _coords(grid)
    X, Y, Z = x[:, None, None], x[None, :, None], x[None, None, :]
    shp = (grid.n,) * 3
    ux = np.broadcast_to(a * np.sin(Z) + c * np.cos(Y), shp)
    uy = np.broadcast_to(b * np.sin(X) + a * np.cos(Z), shp)
    uz = np.broadcast_to(c * np.sin(Y) + b * np.cos(X), shp)
    return [r2c_3d(ux), r2c_3d(uy), r2c_3d(uz)]


def spectral_energy(grid: Grid, u_hat) -> float:
    w = _r2c_weight(grid)
    nt = float(grid.n ** 3)
    return 0.5 * float(sum((w * (c.real ** 2 + c.imag ** 2)).sum() for c in u_hat)) / (nt * nt)


def random_field(grid: Grid, seed: int, amp=1.0):
    """Seeded random spectral field (not Hermitian-cleaned) for parity tests."""
    rng = np.random.default_rng(seed)
    shp = grid.spectral_shape
    return [amp * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) for _ in range(3)]


def hermitian_clean(grid: Grid, u_hat):
    """r2c(c2r(.)): the field a physical-space IC would have produced."""
    shp = (grid.n,) * 3
    return [r2c_3d(c2r_3d(c, shp)) for c in u_hat]
