"""Initial conditions in spectral space (host side, numpy).

The reference builds its ICs on the CPU in physical space and transforms them
with three r2c_3d calls (vonkarman-periodic/src/solver.rs:47-76).  These
generators follow the same contract -- they return ``u_hat`` as three
(n, n, n//2+1) complex128 arrays in the reference layout -- and are the inputs
``Periodic3D`` takes.  Transforms use numpy's pocketfft on the host (set-up
only, not the stepped path).

* ``taylor_green``      -- ic/taylor_green.rs:10-38 (identical field)
* ``abc_flow``          -- ic/abc.rs:14-42 (identical field)
* ``von_karman_isotropic`` -- random isotropic field with the von Karman
  spectrum E(k) ~ (k/kp)^4 / (1 + (k/kp)^2)^(17/6), amplitudes
  sqrt(E(k) / (4 pi k^2)), phases from the reference's xorshift64 stream
  (ic/random_isotropic.rs:31-38, one draw per (ix, iy, iz, c) in C order, DC
  skipped as at :40-43), made Hermitian by r2c(c2r(.)), Leray-projected and
  rescaled to the target energy.  (The reference's own isotropic IC uses
  E ~ k^4 exp(-k^2 / 2 kp^2), ic/random_isotropic.rs:55-58.)
* ``lamb_oseen_tubes``  -- two z-aligned Gaussian-core tubes (circulation +G and
  -G, core radius sigma, separation d about the box centre, centre lines
  displaced in x by eps*sin(z)); omega_z with minimum-image distances, then
  u_hat = i k x omega_hat / |k|^2 (spectral Biot-Savart) and Leray projection.
  (The reference's anti_parallel_tubes writes an x-aligned velocity directly,
  ic/anti_parallel.rs:52-98.)
"""

from __future__ import annotations

import math

import numpy as np

TWO_PI = 2.0 * math.pi
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


# ---------------------------------------------------------------------------
# xorshift64 (ic/random_isotropic.rs:31-38) with GF(2) jump-ahead
# ---------------------------------------------------------------------------

def _xs_step(x: np.ndarray) -> np.ndarray:
    x = x ^ ((x << np.uint64(13)) & _M64)
    x = x ^ (x >> np.uint64(7))
    x = x ^ ((x << np.uint64(17)) & _M64)
    return x


def _matvec(cols: np.ndarray, x: np.ndarray) -> np.ndarray:
    """GF(2) matrix (64 column words) times bit vectors x (any shape)."""
    y = np.zeros_like(x)
    for i in range(64):
        bit = (x >> np.uint64(i)) & np.uint64(1)
        y ^= np.where(bit.astype(bool), cols[i], np.uint64(0))
    return y


def _matmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return _matvec(a, b)  # column j of a.b = a . (column j of b)


def _step_matrix() -> np.ndarray:
    basis = np.array([np.uint64(1) << np.uint64(i) for i in range(64)], dtype=np.uint64)
    return _xs_step(basis)


def _matpow(m: np.ndarray, e: int) -> np.ndarray:
    r = np.array([np.uint64(1) << np.uint64(i) for i in range(64)], dtype=np.uint64)
    while e:
        if e & 1:
            r = _matmul(m, r)
        m = _matmul(m, m)
        e >>= 1
    return r


def xorshift64_stream(seed: int, count: int, lanes: int = 4096) -> np.ndarray:
    """The first ``count`` outputs of the reference's generator as floats in
    [0, 1]: state ^= state << 13; state ^= state >> 7; state ^= state << 17;
    value = state / u64::MAX."""
    if count <= 0:
        return np.zeros(0)
    step = _step_matrix()
    per = -(-count // lanes)
    jump = _matpow(step, per)
    starts = np.empty(lanes, dtype=np.uint64)
    s = _xs_step(np.array([np.uint64(seed)], dtype=np.uint64))  # first output state
    # lane j starts at output j*per: chain jumps in blocks to stay vectorised
    blk = 64
    first = np.empty(blk, dtype=np.uint64)
    cur = s.copy()
    for j in range(blk):
        first[j] = cur[0]
        cur = _matvec(jump, cur)
    jump_blk = _matpow(jump, blk)
    row = first.copy()
    for b in range(0, lanes, blk):
        n = min(blk, lanes - b)
        starts[b:b + n] = row[:n]
        row = _matvec(jump_blk, row)
    out = np.empty((per, lanes), dtype=np.uint64)
    x = starts
    for i in range(per):
        out[i] = x
        x = _xs_step(x)
    flat = out.T.reshape(-1)[:count]
    return flat.astype(np.float64) / float(2 ** 64 - 1)


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def _k(n: int, l: float):
    scale = TWO_PI / l
    kx = np.where(np.arange(n) < n // 2, np.arange(n), np.arange(n) - n).astype(np.float64) * scale
    kz = np.arange(n // 2 + 1, dtype=np.float64) * scale
    return kx[:, None, None], kx[None, :, None], kz[None, None, :]


def _coords(n: int, l: float):
    return np.arange(n, dtype=np.float64) * l / n


def _r2c(x):
    return np.fft.rfftn(x)


def _c2r(xh, n):
    return np.fft.irfftn(xh, s=(n, n, n), axes=(0, 1, 2))


def spectral_energy(u_hat, n: int) -> float:
    w = np.full(n // 2 + 1, 2.0)
    w[0] = 1.0
    w[n // 2] = 1.0
    nt = float(n) ** 3
    return 0.5 * float(sum((w * (c.real ** 2 + c.imag ** 2)).sum() for c in u_hat)) / (nt * nt)


def leray(u_hat, n: int, l: float):
    KX, KY, KZ = _k(n, l)
    k2 = KX * KX + KY * KY + KZ * KZ
    inv = np.where(k2 < 1e-30, 0.0, 1.0 / np.where(k2 < 1e-30, 1.0, k2))
    kd = KX * u_hat[0] + KY * u_hat[1] + KZ * u_hat[2]
    return [u_hat[0] - KX * kd * inv, u_hat[1] - KY * kd * inv, u_hat[2] - KZ * kd * inv]


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------

def taylor_green(n: int, l: float = TWO_PI):
    x = _coords(n, l)
    X, Y, Z = x[:, None, None], x[None, :, None], x[None, None, :]
    shp = (n, n, n)
    ux = np.broadcast_to(np.sin(X) * np.cos(Y) * np.cos(Z), shp)
    uy = np.broadcast_to(-(np.cos(X) * np.sin(Y) * np.cos(Z)), shp)
    return [_r2c(ux), _r2c(uy), _r2c(np.zeros(shp))]


def abc_flow(n: int, a: float = 1.0, b: float = 1.0, c: float = 1.0, l: float = TWO_PI):
    x = _coords(n, l)
    X, Y, Z = x[:, None, None], x[None, :, None], x[None, None, :]
    shp = (n, n, n)
    return [_r2c(np.broadcast_to(a * np.sin(Z) + c * np.cos(Y), shp)),
            _r2c(np.broadcast_to(b * np.sin(X) + a * np.cos(Z), shp)),
            _r2c(np.broadcast_to(c * np.sin(Y) + b * np.cos(X), shp))]


def von_karman_isotropic(n: int, kp: float = 4.0, energy: float = 0.5, seed: int = 42, l: float = TWO_PI):
    """Random isotropic field with the von Karman spectrum, unit-normalised to
    ``energy`` = (1/2)<|u|^2>."""
    KX, KY, KZ = _k(n, l)
    k = np.sqrt(KX * KX + KY * KY + KZ * KZ)
    with np.errstate(divide="ignore", invalid="ignore"):
        ek = (k / kp) ** 4 / (1.0 + (k / kp) ** 2) ** (17.0 / 6.0)
        amp = np.where(k < 1e-10, 0.0, np.sqrt(ek / (4.0 * math.pi * k * k)))
    shp = (n, n, n // 2 + 1)
    nmodes = n * n * (n // 2 + 1)
    draws = xorshift64_stream(seed, 3 * (nmodes - 1))
    ph = np.zeros((nmodes, 3))
    ph[1:] = (2.0 * math.pi * draws).reshape(nmodes - 1, 3)
    u = [amp * np.exp(1j * ph[:, c].reshape(shp)) for c in range(3)]
    u = [_r2c(_c2r(c, n)) for c in u]                 # Hermitian symmetry
    u = leray(u, n, l)
    e = spectral_energy(u, n)
    s = math.sqrt(energy / e) if e > 1e-30 else 1.0
    return [c * s for c in u]


def lamb_oseen_tubes(n: int, circulation: float = 1.0, sigma: float = 0.25, separation: float = 1.0,
                     eps: float = 0.1, l: float = TWO_PI):
    """Anti-parallel z-aligned Lamb-Oseen tubes about the box centre: tube +G at
    y = c - d/2, tube -G at y = c + d/2, both centred at x = c + eps sin(z)."""
    x = _coords(n, l)
    X, Y, Z = x[:, None, None], x[None, :, None], x[None, None, :]
    c = 0.5 * l
    wz = np.zeros((n, n, n))
    amp = circulation / (math.pi * sigma * sigma)
    for sign, yc in ((+1.0, c - 0.5 * separation), (-1.0, c + 0.5 * separation)):
        dx = X - (c + eps * np.sin(TWO_PI * Z / l))
        dy = Y - yc
        dx = dx - l * np.round(dx / l)
        dy = dy - l * np.round(dy / l)
        wz = wz + sign * amp * np.exp(-(dx * dx + dy * dy) / (sigma * sigma))
    w_hat = [np.zeros((n, n, n // 2 + 1), complex), np.zeros((n, n, n // 2 + 1), complex), _r2c(wz)]
    KX, KY, KZ = _k(n, l)
    k2 = KX * KX + KY * KY + KZ * KZ
    inv = np.where(k2 < 1e-30, 0.0, 1.0 / np.where(k2 < 1e-30, 1.0, k2))
    # u_hat = i k x w_hat / k^2
    u = [1j * (KY * w_hat[2] - KZ * w_hat[1]) * inv,
         1j * (KZ * w_hat[0] - KX * w_hat[2]) * inv,
         1j * (KX * w_hat[1] - KY * w_hat[0]) * inv]
    return leray(u, n, l)


def abc_plus_perturbation(n: int, rms: float = 1e-2, kp: float = 8.0, seed: int = 43, l: float = TWO_PI):
    """ABC (A=B=C=1) plus a solenoidal von Karman perturbation with
    sqrt(<|u'|^2>) = rms."""
    base = abc_flow(n, l=l)
    pert = von_karman_isotropic(n, kp=kp, energy=0.5 * rms * rms, seed=seed, l=l)
    return [a + b for a, b in zip(base, pert)]


def project_control(u_hat, n: int, l: float = TWO_PI):
    """Project onto real, divergence-free fields with zero Nyquist entries
    (ix, iy or iz = n/2): with the convention kx[n/2] = -n/2 those entries
    cannot be both Hermitian and divergence-free.  Orthogonal in the L2
    inner product of the physical fields."""
    out = []
    for c in u_hat:
        c = np.array(c, dtype=np.complex128, copy=True)
        c[n // 2, :, :] = 0.0
        c[:, n // 2, :] = 0.0
        c[:, :, n // 2] = 0.0
        out.append(c)
    out = leray(out, n, l)
    return [_r2c(_c2r(c, n)) for c in out]   # Hermitian part on the kz = 0 plane


def solenoidal_direction(n: int, seed: int, kp: float = 4.0, l: float = TWO_PI):
    """Seeded random direction in the control space of the adjoint (real,
    divergence-free, Nyquist-free) with unit L2 norm (<|v|^2> = 1)."""
    v = project_control(von_karman_isotropic(n, kp=kp, energy=0.5, seed=seed, l=l), n, l)
    e = spectral_energy(v, n)
    return [c / np.sqrt(2.0 * e) for c in v]
