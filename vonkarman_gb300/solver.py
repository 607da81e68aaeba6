"""Host-side mirror of vonkarman's API for the periodic step, backed by the
GB300 library.  Names, argument meaning and error behaviour follow the
reference crates:

* ``Periodic3D``    -- vonkarman-periodic/src/solver.rs:12-618 (``Domain`` trait,
                       vonkarman-core/src/domain.rs:39-81)
* ``GpuFftBackend`` -- the ``FftBackend`` trait, vonkarman-fft/src/backend.rs:9-25
* ``create_backend``-- vonkarman-fft/src/select.rs:34-67 (no silent fallback:
                       a missing GPU raises, like ``BackendMode::Cufft``)
* ``energy_spectrum``, ``compensated_spectrum``, ``dissipation_spectrum`` --
                       vonkarman-diag/src/spectrum.rs:13-83
* ``ScalarDiagnostics`` -- vonkarman-diag/src/scalar.rs:6-54
* ``compute_nonlinear`` -- vonkarman-periodic/src/nonlinear.rs:15-39

Spectral arrays are numpy complex128 arrays of shape (n, n, n//2+1) in C order,
exactly the reference's ``Array3<Complex<f64>>``.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat

TWO_PI = 2.0 * math.pi


@dataclass(frozen=True)
class GridSpec:
    """``GridSpec::cubic`` (vonkarman-core/src/field.rs:18-27)."""

    n: int
    l: float = TWO_PI

    @property
    def spectral_shape(self):
        return (self.n, self.n, self.n // 2 + 1)

    @property
    def dx(self) -> float:
        return self.l / self.n

    def padded_3half(self) -> "GridSpec":
        return GridSpec(3 * self.n // 2, self.l)


@dataclass
class SolverOptions:
    """Configuration beyond ``Periodic3D::new(grid, nu, ic, backend)``."""

    precision: str = "fp64"          # "fp64" | "fp32bulk"
    etd_variant: str = "reference"   # "reference" | "cox-matthews"
    integrator: str = "etd-rk4"      # "etd-rk4" | "rk4"
    dt_mode: str = "cfl"             # "cfl" | "fixed"
    dt_fixed: float = 0.0
    cfl_safety: float = 0.5
    device: int = 0


@dataclass
class ScalarDiagnostics:
    time: float
    step: int
    dt: float
    energy: float
    enstrophy: float
    helicity: float
    superhelicity: float
    max_vorticity: float
    energy_dissipation_rate: float
    helicity_dissipation_rate: float
    cfl_number: float

    @classmethod
    def _from_c(cls, t: nat.VkTier1) -> "ScalarDiagnostics":
        return cls(**{f: getattr(t, f) for f, _ in nat.VkTier1._fields_})

    @staticmethod
    def compute_rates(nu: float, enstrophy: float, superhelicity: float):
        """scalar.rs:52-54."""
        return (-2.0 * nu * enstrophy, -2.0 * nu * superhelicity)


def _as_c128(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.shape != tuple(shape):
        raise ValueError(f"expected spectral array of shape {shape}, got {a.shape}")
    return a


class Periodic3D:
    """GPU-resident ``Periodic3D``.

    ``Periodic3D(grid, nu, u_hat, options)`` is ``Periodic3D::new`` with the IC
    already transformed to spectral space (the reference builds it from an
    ``IcType``; here the caller supplies ``u_hat``, see ``vonkarman_gb300.ics``).
    """

    def __init__(self, grid: GridSpec, nu: float, u_hat, options: SolverOptions | None = None, *,
                 _restore=None):
        self.grid = grid
        self.nu = float(nu)
        self.options = options or SolverOptions()
        self._lib = nat.load()
        cfg = nat.VkConfig()
        self._lib.vk_config_default(ctypes.byref(cfg), grid.n, self.nu)
        cfg.lx = cfg.ly = cfg.lz = grid.l
        o = self.options
        cfg.precision = nat.PRECISION[o.precision]
        cfg.etd_variant = nat.ETD_VARIANT[o.etd_variant]
        cfg.integrator = nat.INTEGRATOR[o.integrator]
        cfg.dt_mode = nat.DT_MODE[o.dt_mode]
        cfg.dt_fixed = o.dt_fixed
        cfg.cfl_safety = o.cfl_safety
        cfg.device = o.device
        ctx = ctypes.c_void_p()
        nat.check(self._lib.vk_create(ctypes.byref(cfg), ctypes.byref(ctx)), self._lib, None)
        self._ctx = ctx
        shp = grid.spectral_shape
        comps = [_as_c128(c, shp) for c in u_hat]
        if _restore is None:
            nat.check(self._lib.vk_set_state_host(ctx, *[nat.dptr(c) for c in comps]), self._lib, ctx)
        else:
            time, step, dt = _restore
            nat.check(self._lib.vk_restore_host(ctx, *[nat.dptr(c) for c in comps], float(time), int(step),
                                                float(dt)), self._lib, ctx)

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.vk_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, fn, *args):
        nat.check(fn(self._ctx, *args), self._lib, self._ctx)

    # -- checkpoint (solver.rs:111-159) ------------------------------------
    def checkpoint_data(self) -> dict:
        return dict(u_hat=self.u_hat(), time=self.time(), step_count=self.step_count(), dt=self.dt(),
                    grid=self.grid, nu=self.nu)

    @classmethod
    def from_checkpoint(cls, data: dict, options: SolverOptions | None = None) -> "Periodic3D":
        return cls(data["grid"], data["nu"], data["u_hat"], options,
                   _restore=(data["time"], data["step_count"], data["dt"]))

    # -- Domain trait -----------------------------------------------------
    def step(self, nsteps: int = 1):
        self._call(self._lib.vk_step, int(nsteps))

    def use_graphs(self, enable: bool = True):
        """Replay steps as captured CUDA graphs (the default) or launch every
        kernel eagerly."""
        self._call(self._lib.vk_use_graphs, 1 if enable else 0)

    def _scalar(self, fn) -> float:
        v = ctypes.c_double()
        self._call(fn, ctypes.byref(v))
        return v.value

    def time(self) -> float:
        return self._scalar(self._lib.vk_time)

    def dt(self) -> float:
        return self._scalar(self._lib.vk_dt)

    def step_count(self) -> int:
        v = ctypes.c_uint64()
        self._call(self._lib.vk_step_count, ctypes.byref(v))
        return int(v.value)

    def cfl_dt(self) -> float:
        return self._scalar(self._lib.vk_cfl_dt)

    def energy(self) -> float:
        return self._scalar(self._lib.vk_energy)

    def enstrophy(self) -> float:
        return self._scalar(self._lib.vk_enstrophy)

    def helicity(self) -> float:
        return self._scalar(self._lib.vk_helicity)

    def superhelicity(self) -> float:
        return self._scalar(self._lib.vk_superhelicity)

    def max_vorticity(self) -> float:
        return self._scalar(self._lib.vk_max_vorticity)

    def tier1(self) -> ScalarDiagnostics:
        t = nat.VkTier1()
        self._call(self._lib.vk_tier1, ctypes.byref(t))
        return ScalarDiagnostics._from_c(t)

    def u_hat(self):
        shp = self.grid.spectral_shape
        out = [np.empty(shp, dtype=np.complex128) for _ in range(3)]
        self._call(self._lib.vk_get_state_host, *[nat.dptr(c) for c in out])
        return out

    def set_fused_diagnostics(self, tier1_every: int = 0, spectrum_every: int = 0):
        """Accumulate the Tier-1 sums / shell spectrum inside the final stage of
        every step whose count is a multiple of the given cadence (0: off);
        ``tier1()`` / ``energy_spectrum()`` on such a state then skip their own
        pass over it."""
        self._call(self._lib.vk_set_fused_diagnostics, int(tier1_every), int(spectrum_every))

    def run(self, nsteps: int, every: int = 1):
        """Advance nsteps steps, recording Tier-1 after every ``every``-th step
        (one device->host transfer at the end)."""
        nrec = nsteps // every if every > 0 else 0
        buf = (nat.VkTier1 * max(nrec, 1))()
        got = ctypes.c_int64()
        self._call(self._lib.vk_run, int(nsteps), int(every), buf, int(nrec), ctypes.byref(got))
        return [ScalarDiagnostics._from_c(buf[i]) for i in range(got.value)]


    # -- discrete adjoint (autograd-Function pattern) -------------------------
    ADJ_SCHEDULES = {"two-level": 0, "binomial": 1}

    def adjoint_forward(self, nsteps: int, nsnap: int = 20, schedule: str = "two-level") -> float:
        """Run nsteps fixed-dt steps keeping nsnap checkpoints; returns
        J = final enstrophy.  The state advances.  schedule: "two-level"
        (nsnap segment checkpoints, one recompute pass storing each segment's
        stage inputs) or "binomial" (nsnap state slots reversed by the
        treeverse schedule: less memory, more recomputation)."""
        if schedule not in self.ADJ_SCHEDULES:
            raise ValueError(f"schedule must be one of {sorted(self.ADJ_SCHEDULES)}")
        self._call(self._lib.vk_adjoint_set_schedule, self.ADJ_SCHEDULES[schedule])
        v = ctypes.c_double()
        self._call(self._lib.vk_adjoint_forward, int(nsteps), int(nsnap), ctypes.byref(v))
        return v.value

    def adjoint_backward(self):
        """dJ/du_0 of the preceding adjoint_forward, in the L2 inner product of
        the physical fields, projected on real divergence-free Nyquist-free
        fields."""
        shp = self.grid.spectral_shape
        out = [np.empty(shp, dtype=np.complex128) for _ in range(3)]
        self._call(self._lib.vk_adjoint_backward, *[nat.dptr(c) for c in out])
        return out

    # -- measurement ----------------------------------------------------------
    def step_timed(self, nsteps: int) -> float:
        """Enqueue nsteps steps between two CUDA events on the context's
        stream; returns the device milliseconds between them."""
        v = ctypes.c_double()
        self._call(self._lib.vk_step_timed, int(nsteps), ctypes.byref(v))
        return v.value

    def event_mark(self, slot: int):
        self._call(self._lib.vk_event_mark, int(slot))

    def event_elapsed(self, a: int, b: int) -> float:
        v = ctypes.c_double()
        self._call(self._lib.vk_event_elapsed, int(a), int(b), ctypes.byref(v))
        return v.value

    def profile(self, enable: bool = True):
        self._call(self._lib.vk_profile_enable, 1 if enable else 0)

    def profile_read(self) -> dict:
        """{pass name: (total ms, launches)} since profiling was enabled."""
        n = nat.NPASS
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        self._call(self._lib.vk_profile_read, ms, cnt, n)
        return {self._lib.vk_profile_pass_name(i).decode(): (ms[i], int(cnt[i])) for i in range(n)}

    def restore_state(self, u_hat, time: float, step_count: int, dt: float):
        """Upload a state in place (Periodic3D::from_checkpoint on this context)."""
        shp = self.grid.spectral_shape
        comps = [_as_c128(c, shp) for c in u_hat]
        self._call(self._lib.vk_restore_host, *[nat.dptr(c) for c in comps], float(time), int(step_count),
                   float(dt))


def probe_fma_peak(device: int = 0, fp64: bool = True) -> float:
    """Measured FMA throughput of the device (GFLOP/s)."""
    lib = nat.load()
    v = ctypes.c_double()
    nat.check(lib.vk_probe_fma_peak(int(device), 1 if fp64 else 0, ctypes.byref(v)), lib, None)
    return v.value


def energy_spectrum(solver: Periodic3D):
    """(shells, E(k)) of the solver's current state (spectrum.rs:13-60)."""
    lib = solver._lib
    n = ctypes.c_int32()
    nat.check(lib.vk_spectrum_len(solver._ctx, ctypes.byref(n)), lib, solver._ctx)
    shells = np.empty(n.value)
    spec = np.empty(n.value)
    nat.check(lib.vk_spectrum(solver._ctx, nat.dptr(shells), nat.dptr(spec), n.value), lib, solver._ctx)
    return shells, spec


def compensated_spectrum(shells, spectrum):
    """k^{5/3} E(k) (spectrum.rs:66-72)."""
    shells = np.asarray(shells, dtype=np.float64)
    return np.where(shells > 0.0, np.power(shells, 5.0 / 3.0) * np.asarray(spectrum), 0.0)


def dissipation_spectrum(shells, spectrum, nu: float):
    """2 nu k^2 E(k) (spectrum.rs:77-83)."""
    shells = np.asarray(shells, dtype=np.float64)
    return 2.0 * nu * shells * shells * np.asarray(spectrum)


def compute_nonlinear(solver: Periodic3D, u_hat):
    """N_hat = P[F(u x omega)] of ``u_hat`` on the solver's grid (nonlinear.rs:15-39)."""
    lib = solver._lib
    shp = solver.grid.spectral_shape
    ins = [_as_c128(c, shp) for c in u_hat]
    outs = [np.empty(shp, dtype=np.complex128) for _ in range(3)]
    nat.check(lib.vk_nonlinear_host(solver._ctx, *[nat.dptr(c) for c in ins], *[nat.dptr(c) for c in outs]),
              lib, solver._ctx)
    return outs


@dataclass
class SpectralOps:
    """The public fields of ``SpectralOps`` (vonkarman-core/src/spectral_ops.rs:10-22),
    as the GPU forms them: ``kx``, ``ky`` (n), ``kz`` (n//2+1), ``k_mag_sq``
    ((n, n, n//2+1)), bit-identical to ``SpectralOps::new``."""

    kx: np.ndarray
    ky: np.ndarray
    kz: np.ndarray
    k_mag_sq: np.ndarray
    grid: GridSpec


def spectral_ops(solver: Periodic3D) -> SpectralOps:
    """``SpectralOps`` of the solver's grid (spectral_ops.rs:26-74)."""
    lib = solver._lib
    n = solver.grid.n
    kx, ky, kz = np.empty(n), np.empty(n), np.empty(n // 2 + 1)
    k2 = np.empty(solver.grid.spectral_shape)
    nat.check(lib.vk_wavenumbers(solver._ctx, nat.dptr(kx), nat.dptr(ky), nat.dptr(kz), nat.dptr(k2)), lib,
              solver._ctx)
    return SpectralOps(kx, ky, kz, k2, solver.grid)


def apply_viscous(solver: Periodic3D, u_hat, nu: float):
    """``SpectralOps::apply_viscous`` (spectral_ops.rs:154-175): -(nu |k|^2) u_hat
    per component, on the GPU in the solver's precision."""
    lib = solver._lib
    shp = solver.grid.spectral_shape
    ins = [_as_c128(c, shp) for c in u_hat]
    outs = [np.empty(shp, dtype=np.complex128) for _ in range(3)]
    nat.check(lib.vk_apply_viscous_host(solver._ctx, float(nu), *[nat.dptr(c) for c in ins],
                                        *[nat.dptr(c) for c in outs]), lib, solver._ctx)
    return outs


def nonlinear_adjoint(solver: Periodic3D, x, nbar):
    """N'(x)^T nbar in the raw Euclidean inner product of the stored entries."""
    lib = solver._lib
    shp = solver.grid.spectral_shape
    xs = [_as_c128(c, shp) for c in x]
    bs = [_as_c128(c, shp) for c in nbar]
    outs = [np.empty(shp, dtype=np.complex128) for _ in range(3)]
    nat.check(lib.vk_nonlinear_adjoint_host(solver._ctx, *[nat.dptr(c) for c in xs], *[nat.dptr(c) for c in bs],
                                            *[nat.dptr(c) for c in outs]), lib, solver._ctx)
    return outs


def l2_inner(a, b, n: int) -> float:
    """<a, b> = sum w Re(conj(a) b) / N^6, the L2 inner product of the physical
    fields (R2C weights w = 1 at iz in {0, n/2}, else 2)."""
    w = np.full(n // 2 + 1, 2.0)
    w[0] = w[n // 2] = 1.0
    nt2 = float(n) ** 6
    return float(sum((w * (np.conj(x) * y).real).sum() for x, y in zip(a, b))) / nt2


class GpuFftBackend:
    """``FftBackend<f64>`` on the GPU (backend.rs:9-25).  ``r2c_3d`` is the
    unnormalised forward transform; ``c2r_3d`` includes 1/(nx ny nz)."""

    def __init__(self, nx: int, ny: int, nz: int, precision: str = "fp64", device: int = 0):
        self._lib = nat.load()
        self.shape = (nx, ny, nz)
        h = ctypes.c_void_p()
        nat.check(self._lib.vk_fft_create(nx, ny, nz, nat.PRECISION[precision], device, ctypes.byref(h)),
                  self._lib, None)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.vk_fft_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def r2c_3d(self, x) -> np.ndarray:
        nx, ny, nz = self.shape
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != self.shape:
            raise ValueError(f"expected {self.shape}, got {x.shape}")
        out = np.empty((nx, ny, nz // 2 + 1), dtype=np.complex128)
        nat.check(self._lib.vk_fft_r2c_host(self._h, nat.dptr(x), nat.dptr(out)), self._lib, fft=self._h)
        return out

    def c2r_3d(self, xh) -> np.ndarray:
        nx, ny, nz = self.shape
        xh = _as_c128(xh, (nx, ny, nz // 2 + 1))
        out = np.empty(self.shape, dtype=np.float64)
        nat.check(self._lib.vk_fft_c2r_host(self._h, nat.dptr(xh), nat.dptr(out)), self._lib, fft=self._h)
        return out

    def name(self) -> str:
        return self._lib.vk_fft_name(self._h).decode()

    def precision_digits(self) -> int:
        return int(self._lib.vk_fft_precision_digits(self._h))


def create_backend(nx: int, ny: int, nz: int, mode: str = "native") -> GpuFftBackend:
    """``create_backend`` with a native GPU mode (select.rs:34-67).  Only the
    native mode exists here; any other mode is rejected rather than silently
    falling back to a CPU path."""
    if mode.lower() not in ("native", "gpu", "cuda", "auto"):
        raise ValueError(f"backend mode {mode!r} is not provided by vonkarman_gb300")
    return GpuFftBackend(nx, ny, nz)
