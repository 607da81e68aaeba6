"""ctypes wrapper of the oracle's C restatement (oracle/vk_cpu.c).

TEST AND BENCHMARK INFRASTRUCTURE ONLY: the timed CPU baseline of bench.py
and a cross-check of the numpy oracle.  The product never imports this.
"""

from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import build_cpu

_lib = None
_DP = ctypes.POINTER(ctypes.c_double)


def load():
    global _lib
    if _lib is None:
        path = build_cpu.build()
        if path is None:
            raise RuntimeError("oracle/vk_cpu.c is missing")
        lib = ctypes.CDLL(path)
        lib.vkc_create.restype = ctypes.c_void_p
        lib.vkc_create.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double]
        lib.vkc_destroy.argtypes = [ctypes.c_void_p]
        lib.vkc_set_state.argtypes = [ctypes.c_void_p, _DP, _DP, _DP]
        lib.vkc_get_state.argtypes = [ctypes.c_void_p, _DP, _DP, _DP]
        lib.vkc_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.vkc_nonlinear.argtypes = [ctypes.c_void_p, _DP, _DP, _DP, _DP, _DP, _DP]
        lib.vkc_time.restype = ctypes.c_double
        lib.vkc_time.argtypes = [ctypes.c_void_p]
        lib.vkc_dt.restype = ctypes.c_double
        lib.vkc_dt.argtypes = [ctypes.c_void_p]
        lib.vkc_set_threads.argtypes = [ctypes.c_int]
        lib.vkc_max_threads.restype = ctypes.c_int
        lib.vkc_r2c_3d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP, _DP]
        lib.vkc_c2r_3d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP, _DP]
        lib.vkc_set_cufft.argtypes = [ctypes.c_int]
        lib.vkc_cufft_error.restype = ctypes.c_char_p
        lib.vkc_uses_cufft.argtypes = [ctypes.c_void_p]
        lib.vkc_spectrum.argtypes = [ctypes.c_void_p, _DP, ctypes.c_int]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(_DP)


def set_threads(t: int):
    load().vkc_set_threads(int(t))


def max_threads() -> int:
    return int(load().vkc_max_threads())


def set_cufft(on: bool):
    """Route the 3-D transforms of solvers created afterwards through the
    reference's cuFFT backend pattern (vonkarman-fft/src/cufft.rs: per-call
    host <-> device copies around cufftExecD2Z / Z2D, host normalisation).
    Raises RuntimeError when libcudart / libcufft cannot be loaded."""
    lib = load()
    if lib.vkc_set_cufft(1 if on else 0) != 0:
        raise RuntimeError(lib.vkc_cufft_error().decode(errors="replace"))


class CpuSolver:
    """Periodic3D on the CPU restatement (ETD-RK4 reference variant)."""

    def __init__(self, n, nu, u_hat, dt_mode="cfl", dt_fixed=0.0, cfl_safety=0.5, l=2.0 * math.pi):
        self.lib = load()
        self.n = n
        self.h = self.lib.vkc_create(n, l, nu, 1 if dt_mode == "fixed" else 0, dt_fixed, cfl_safety)
        if not self.h:
            raise ValueError("bad grid")
        comps = [np.ascontiguousarray(c, dtype=np.complex128) for c in u_hat]
        self.lib.vkc_set_state(self.h, *[_p(c) for c in comps])

    def step(self, k=1):
        self.lib.vkc_step(self.h, int(k))

    def u_hat(self):
        shp = (self.n, self.n, self.n // 2 + 1)
        out = [np.empty(shp, np.complex128) for _ in range(3)]
        self.lib.vkc_get_state(self.h, *[_p(c) for c in out])
        return out

    def nonlinear(self, u_hat):
        shp = (self.n, self.n, self.n // 2 + 1)
        ins = [np.ascontiguousarray(c, dtype=np.complex128) for c in u_hat]
        out = [np.empty(shp, np.complex128) for _ in range(3)]
        self.lib.vkc_nonlinear(self.h, *[_p(c) for c in ins], *[_p(c) for c in out])
        return out

    def spectrum(self):
        """energy_spectrum of the current state (spectrum.rs:13-60)."""
        kmx = float(self.n // 2)
        nsh = int(math.ceil(math.sqrt(3.0 * kmx * kmx))) + 1
        out = np.empty(nsh)
        self.lib.vkc_spectrum(self.h, _p(out), nsh)
        return out

    def uses_cufft(self) -> bool:
        return bool(self.lib.vkc_uses_cufft(self.h))

    def time(self):
        return self.lib.vkc_time(self.h)

    def dt(self):
        return self.lib.vkc_dt(self.h)

    def close(self):
        if self.h:
            self.lib.vkc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def r2c_3d(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    nx, ny, nz = x.shape
    out = np.empty((nx, ny, nz // 2 + 1), np.complex128)
    load().vkc_r2c_3d(nx, ny, nz, _p(x), _p(out))
    return out


def c2r_3d(xh, shape):
    xh = np.ascontiguousarray(xh, dtype=np.complex128)
    out = np.empty(shape, np.float64)
    load().vkc_c2r_3d(*shape, _p(xh), _p(out))
    return out
