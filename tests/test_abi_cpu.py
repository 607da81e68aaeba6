"""CPU-only checks of the C-ABI boundary: the shared library loads, exports
every symbol include/vonkarman_gpu.h declares, and rejects invalid
configurations with status codes before touching a device.  No compute
calls are made here."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vonkarman_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vk_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from vonkarman_gb300 import build

    build.build()
    from vonkarman_gb300 import _native

    return _native.load()


def test_header_declares_expected_entry_points():
    syms = declared_symbols()
    for s in ("vk_create", "vk_step", "vk_tier1", "vk_spectrum", "vk_fft_r2c_host", "vk_fft_c2r_host",
              "vk_set_state_host", "vk_get_state_host", "vk_restore_host", "vk_nonlinear_host", "vk_run"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(lib):
    from vonkarman_gb300 import _native

    assert set(declared_symbols()) <= set(_native.SIGNATURES)


def test_abi_version(lib):
    assert lib.vk_abi_version() == 1


def _cfg(lib, n=16, nu=0.01):
    from vonkarman_gb300 import _native as nat

    c = nat.VkConfig()
    lib.vk_config_default(ctypes.byref(c), n, nu)
    return c


def test_config_default_matches_reference_defaults(lib):
    c = _cfg(lib, 32, 0.02)
    assert (c.nx, c.ny, c.nz) == (32, 32, 32)
    assert abs(c.lx - 2 * 3.141592653589793) < 1e-15
    assert c.cfl_safety == 0.5  # solver.rs:89
    assert c.precision == 0 and c.dt_mode == 0 and c.integrator == 0 and c.etd_variant == 0


@pytest.mark.parametrize("mutate,code", [
    (lambda c: setattr(c, "nx", 12), 2),          # non-cubic
    (lambda c: (setattr(c, "nx", 24), setattr(c, "ny", 24), setattr(c, "nz", 24)), 1),  # not 2^k
    (lambda c: (setattr(c, "nx", 4), setattr(c, "ny", 4), setattr(c, "nz", 4)), 1),     # < 8
    (lambda c: setattr(c, "nu", 0.0), 1),
    (lambda c: setattr(c, "nu", -1.0), 1),
    (lambda c: setattr(c, "lx", -1.0), 1),
    (lambda c: setattr(c, "precision", 7), 1),
    (lambda c: setattr(c, "cfl_safety", 1.5), 1),
    (lambda c: setattr(c, "cfl_safety", 0.0), 1),
    (lambda c: (setattr(c, "dt_mode", 1), setattr(c, "dt_fixed", 0.0)), 1),
    (lambda c: setattr(c, "integrator", 3), 1),
])
def test_invalid_configs_rejected(lib, mutate, code):
    c = _cfg(lib)
    mutate(c)
    ctx = ctypes.c_void_p()
    assert lib.vk_create(ctypes.byref(c), ctypes.byref(ctx)) == code
    assert not ctx.value
    assert lib.vk_last_error(None)


def test_fft_invalid_lengths_rejected(lib):
    h = ctypes.c_void_p()
    assert lib.vk_fft_create(10, 16, 16, 0, 0, ctypes.byref(h)) == 2
    assert lib.vk_fft_create(16, 16, 1024, 0, 0, ctypes.byref(h)) == 2
    assert lib.vk_fft_create(16, 16, 16, 5, 0, ctypes.byref(h)) == 1


def test_null_arguments(lib):
    assert lib.vk_create(None, None) == 1
    assert lib.vk_step(None, 1) == 1
    assert lib.vk_destroy(None) == 0
    assert lib.vk_spectral_len(None) == -1
    assert lib.vk_adjoint_set_schedule(None, 0) == 1
    assert lib.vk_adjoint_forward(None, 10, 2, None) == 1
    assert lib.vk_adjoint_backward(None, None, None, None) == 1
