"""The algorithmic traffic model behind bench.py's GB/s and roofline figures:
per-pass element counts of one nonlinear evaluation (units of N^2 H complex
elements) and the step total with the CFL pass."""

import math

import pytest

bench = pytest.importorskip("bench")


@pytest.mark.parametrize("n", [64, 256, 512])
def test_pass_model_element_counts(n):
    h, m = n // 2 + 1, 3 * n // 2
    unit = n * n * h
    mdl = bench.pass_model(n)
    # reads + writes per pass, in N^2 H units (M/N = 3/2)
    want = {
        "P1_x_inverse_pad_curl": 3 + 5 * 1.5,          # R u (3), W 5 fields (M, N, H)
        "P2_y_inverse_pad_omega": 5 * 1.5 + 6 * 2.25,  # R 5 x (M, N, H), W 6 x (M, M, H)
        "P3_z_c2r_cross_r2c": 9 * 2.25,                # R 6, W 3 x (M, M, H)
        "P4_y_forward_trunc": 3 * 2.25 + 3 * 1.5,      # R 3 x (M, M, H), W 3 x (M, N, H)
        "P5_x_forward_trunc_leray_stage": 3 * 1.5 + 11.25,  # R 3 x (M, N, H) + stage epilogue mean
        "NX_ngrid_x_inverse": 6,
        "NY_ngrid_y_inverse": 6,
        "NZ_ngrid_z_c2r_max": 3,
    }
    for k, units in want.items():
        assert mdl[k][0] == pytest.approx(units * unit, rel=1e-12), k
    assert m * m * h == pytest.approx(2.25 * unit)


def test_stage_epilogue_mean_counts_the_state_read():
    # ETD stages: (R u W n1,temp), (R u,n1 W acc,temp), (R u,n1,acc W acc,temp), (R u,acc W u)
    per_stage = [3 + 6, 6 + 6, 9 + 6, 6 + 3]
    assert sum(per_stage) / 4 == 11.25


@pytest.mark.parametrize("elem", [8, 16])
def test_step_bytes_is_330_units(elem):
    n = 256
    unit = n * n * (n // 2 + 1)
    assert bench.step_bytes(n, elem) == pytest.approx(330 * unit * elem, rel=1e-12)
    assert math.isclose(bench.step_bytes(n, 8) / 1e9, 22.3, rel_tol=0.01)
