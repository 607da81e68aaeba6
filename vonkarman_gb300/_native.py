"""ctypes binding of libvonkarman_gpu.so (the C ABI in include/vonkarman_gpu.h).

The library must exist; there is no fallback.  ``load()`` raises if the
shared object is missing or does not export the expected ABI version.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint64, c_void_p

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libvonkarman_gpu.so")
ABI_VERSION = 1
NPASS = 20

VK_OK = 0
STATUS_NAMES = {0: "VK_OK", 1: "VK_ERR_INVALID", 2: "VK_ERR_UNSUPPORTED", 3: "VK_ERR_CUDA",
                4: "VK_ERR_OOM", 5: "VK_ERR_STATE", 6: "VK_ERR_NONFINITE"}

PRECISION = {"fp64": 0, "fp32bulk": 1}
ETD_VARIANT = {"reference": 0, "cox-matthews": 1}
INTEGRATOR = {"etd-rk4": 0, "rk4": 1}
DT_MODE = {"cfl": 0, "fixed": 1}


class VkConfig(ctypes.Structure):
    _fields_ = [("nx", c_int32), ("ny", c_int32), ("nz", c_int32),
                ("lx", c_double), ("ly", c_double), ("lz", c_double),
                ("nu", c_double),
                ("precision", c_int32), ("etd_variant", c_int32), ("integrator", c_int32), ("dt_mode", c_int32),
                ("dt_fixed", c_double), ("cfl_safety", c_double),
                ("device", c_int32), ("reserved", c_int32)]


class VkTier1(ctypes.Structure):
    _fields_ = [("time", c_double), ("step", c_uint64), ("dt", c_double), ("energy", c_double),
                ("enstrophy", c_double), ("helicity", c_double), ("superhelicity", c_double),
                ("max_vorticity", c_double), ("energy_dissipation_rate", c_double),
                ("helicity_dissipation_rate", c_double), ("cfl_number", c_double)]


_DP = POINTER(c_double)
_CTX = c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "vk_abi_version": (c_int, []),
    "vk_last_error": (c_char_p, [_CTX]),
    "vk_config_default": (None, [POINTER(VkConfig), c_int32, c_double]),
    "vk_create": (c_int, [POINTER(VkConfig), POINTER(_CTX)]),
    "vk_destroy": (c_int, [_CTX]),
    "vk_spectral_len": (c_int64, [_CTX]),
    "vk_set_state_host": (c_int, [_CTX, _DP, _DP, _DP]),
    "vk_restore_host": (c_int, [_CTX, _DP, _DP, _DP, c_double, c_uint64, c_double]),
    "vk_get_state_host": (c_int, [_CTX, _DP, _DP, _DP]),
    "vk_step": (c_int, [_CTX, c_int64]),
    "vk_use_graphs": (c_int, [_CTX, c_int32]),
    "vk_time": (c_int, [_CTX, _DP]),
    "vk_step_count": (c_int, [_CTX, POINTER(c_uint64)]),
    "vk_dt": (c_int, [_CTX, _DP]),
    "vk_cfl_dt": (c_int, [_CTX, _DP]),
    "vk_tier1": (c_int, [_CTX, POINTER(VkTier1)]),
    "vk_energy": (c_int, [_CTX, _DP]),
    "vk_enstrophy": (c_int, [_CTX, _DP]),
    "vk_helicity": (c_int, [_CTX, _DP]),
    "vk_superhelicity": (c_int, [_CTX, _DP]),
    "vk_max_vorticity": (c_int, [_CTX, _DP]),
    "vk_run": (c_int, [_CTX, c_int64, c_int64, POINTER(VkTier1), c_int64, POINTER(c_int64)]),
    "vk_set_fused_diagnostics": (c_int, [_CTX, c_int64, c_int64]),
    "vk_spectrum_len": (c_int, [_CTX, POINTER(c_int32)]),
    "vk_spectrum": (c_int, [_CTX, _DP, _DP, c_int32]),
    "vk_nonlinear_host": (c_int, [_CTX, _DP, _DP, _DP, _DP, _DP, _DP]),
    "vk_apply_viscous_host": (c_int, [_CTX, c_double, _DP, _DP, _DP, _DP, _DP, _DP]),
    "vk_wavenumbers": (c_int, [_CTX, _DP, _DP, _DP, _DP]),
    "vk_adjoint_forward": (c_int, [_CTX, c_int64, c_int32, _DP]),
    "vk_adjoint_set_schedule": (c_int, [_CTX, c_int32]),
    "vk_adjoint_backward": (c_int, [_CTX, _DP, _DP, _DP]),
    "vk_nonlinear_adjoint_host": (c_int, [_CTX, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
    "vk_step_timed": (c_int, [_CTX, c_int64, _DP]),
    "vk_profile_enable": (c_int, [_CTX, c_int32]),
    "vk_profile_read": (c_int, [_CTX, _DP, POINTER(c_int64), c_int32]),
    "vk_profile_pass_name": (c_char_p, [c_int32]),
    "vk_probe_fma_peak": (c_int, [c_int32, c_int32, _DP]),
    "vk_stream": (c_int, [_CTX, POINTER(c_void_p)]),
    "vk_event_mark": (c_int, [_CTX, c_int32]),
    "vk_event_elapsed": (c_int, [_CTX, c_int32, c_int32, _DP]),
    "vk_pinned_alloc": (c_int, [ctypes.c_size_t, POINTER(c_void_p)]),
    "vk_pinned_free": (c_int, [c_void_p]),
    "vk_spectrum_noalloc": (c_int, [c_void_p, c_int32, c_double, c_int32, c_void_p, c_void_p]),
    "vk_fft_create": (c_int, [c_int32, c_int32, c_int32, c_int32, c_int32, POINTER(c_void_p)]),
    "vk_fft_destroy": (c_int, [c_void_p]),
    "vk_fft_last_error": (c_char_p, [c_void_p]),
    "vk_fft_r2c_host": (c_int, [c_void_p, _DP, _DP]),
    "vk_fft_c2r_host": (c_int, [c_void_p, _DP, _DP]),
    "vk_fft_r2c_device": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "vk_fft_c2r_device": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "vk_fft_name": (c_char_p, [c_void_p]),
    "vk_fft_precision_digits": (c_int, [c_void_p]),
}

_lib = None


def load(path: str | None = None):
    """Load the shared library once and bind every symbol of the ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(vonkarman_gb300/build.py); there is no CPU fallback")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.vk_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{p}: ABI version {lib.vk_abi_version()} != {ABI_VERSION}")
    if path is None:
        _lib = lib
    return lib


class VkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(code: int, lib, ctx=None, fft=None):
    if code != VK_OK:
        if fft is not None:
            msg = lib.vk_fft_last_error(fft)
        else:
            msg = lib.vk_last_error(ctx)
        raise VkError(code, (msg or b"").decode(errors="replace"))


def dptr(a):
    return a.ctypes.data_as(_DP)
