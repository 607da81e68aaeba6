"""Binomial checkpoint schedule (vonkarman_gb300/csrc/vk_schedule.h) on the
CPU: a simulated executor whose states are step indices checks that every
step is reversed exactly once, last first, from the right state; that no
more than nsnap slots hold a state at once; and that the forward work stays
within r sweeps of the chain (r the least with C(nsnap - 1 + r, r) >= nsteps)."""

import math
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [(1, 1), (2, 1), (7, 1), (10, 2), (20, 3), (100, 5), (1000, 20), (1000, 60), (997, 7), (64, 64),
         (5000, 10)]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("sched") / "schedule_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "vonkarman_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "schedule_check.cpp"), "-o", exe], check=True)
    return exe


def test_treeverse_reverses_every_step_within_slots_and_sweeps(checker):
    args = [str(v) for case in CASES for v in case]
    out = subprocess.run([checker, *args], check=True, capture_output=True, text=True).stdout.split("\n")
    for (nsteps, nsnap), line in zip(CASES, out):
        f = line.split()
        assert f[0] == "ok", line
        adv, slots, r, adv_pre, spine_last = int(f[2]), int(f[3]), int(f[4]), int(f[5]), int(f[6])
        assert slots <= nsnap
        assert nsnap == 1 or math.comb(nsnap - 1 + r, r) >= nsteps
        # every step is advanced at most r times in the reversal sweeps
        assert adv <= r * nsteps, (nsteps, nsnap, adv, r)
        # with the first descent stored by the forward run, the reversal skips
        # exactly the advances that reached its last checkpoint
        assert adv_pre == adv - spine_last, (nsteps, nsnap, adv, adv_pre, spine_last)
        if nsnap > 1 and nsteps > 1:
            assert spine_last >= 1


def test_binomial_1000_steps_20_slots_advances(checker):
    """The schedule of the checkpointed-adjoint workload (1000 steps, 20 state
    slots): 2806 advances in the reversal, 1807 once the forward run has
    stored the first descent, with every step advanced at most r = 3 times;
    Griewank's lower bound for 19 free slots, r * l - C(s + r, r - 1) = 2769,
    is within 2 % of the unstored count."""
    out = subprocess.run([checker, "1000", "20"], check=True, capture_output=True, text=True).stdout.split()
    assert out[0] == "ok"
    adv, r, adv_pre = int(out[2]), int(out[4]), int(out[5])
    assert (adv, adv_pre, r) == (2806, 1807, 3)
    bound = r * 1000 - math.comb(19 + r, r - 1)
    assert bound == 2769 and bound <= adv <= 1.02 * bound
