"""The allocation-free spectrum entry point, through the C ABI.

vk_spectrum_noalloc is for callers that cannot allocate device memory (graph
capture, a framework allocator that owns the device, latency-critical loops):
they hand in a state they already hold on the device and an output buffer,
and the library uses a fixed scratch array instead of cudaMalloc.  This test
compares it with vk_spectrum (which runs on a solver context) on two calls in
a row, since every call shares and overwrites the same scratch."""

import ctypes
import math

import numpy as np
import pytest

from oracle import vk_oracle as vo

pytestmark = pytest.mark.gpu

TOL_DIAG = 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp32bulk"])
def test_spectrum_noalloc_matches_vk_spectrum(precision):
    """Both precisions: the FP32-bulk state is handed over as the complex64
    values the solver holds (an exact round trip through the FP64 host copy),
    so both entry points form the same FP32 per-mode products and differ only
    in the order of their FP64 sums."""
    torch = pytest.importorskip("torch")
    import vonkarman_gb300 as vk
    from vonkarman_gb300 import _native as nat

    lib = nat.load()
    code = nat.PRECISION[precision]
    for n, seed in ((32, 21), (64, 22)):
        g = vo.Grid(n)
        u0 = vo.hermitian_clean(g, vo.random_field(g, seed, amp=float(n) ** 3 / 50.0))
        s = vk.Periodic3D(vk.GridSpec(n), 0.01, u0, vk.SolverOptions(precision=precision))
        s.step(2)
        _, want = vk.energy_spectrum(s)
        state = np.ascontiguousarray(np.stack(s.u_hat()))
        s.close()
        if precision == "fp32bulk":
            state = state.astype(np.complex64)
        dev_u = torch.from_numpy(state).to("cuda")
        out = torch.empty(len(want), dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = lib.vk_spectrum_noalloc(ctypes.c_void_p(dev_u.data_ptr()), n, 2.0 * math.pi, code,
                                         ctypes.c_void_p(out.data_ptr()), None)
            assert rc == 0, lib.vk_last_error(None)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert np.abs(got - want).max() <= TOL_DIAG * np.abs(want).max()


def test_spectrum_noalloc_rejects_sizes_beyond_its_scratch():
    from vonkarman_gb300 import _native as nat

    lib = nat.load()
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.vk_spectrum_noalloc(fake, 1024, 2.0 * math.pi, 0, fake, None) == 2
    assert b"512" in lib.vk_last_error(None)
    assert lib.vk_spectrum_noalloc(fake, 24, 2.0 * math.pi, 0, fake, None) == 1
