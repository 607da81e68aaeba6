"""Host-side logic on the CPU: the seeded generator behind the synthetic
workloads, the initial-condition generators' invariants, and the run-loop
helpers (stop rule of the reference's run loop, interpolation to t_end)."""

import math
from types import SimpleNamespace

import numpy as np
import pytest

from vonkarman_gb300 import ics

MASK = (1 << 64) - 1


def xorshift64_scalar(seed, count):
    x, out = seed, []
    for _ in range(count):
        x ^= (x << 13) & MASK
        x ^= x >> 7
        x ^= (x << 17) & MASK
        out.append(x / float(MASK))
    return np.array(out)


@pytest.mark.parametrize("seed,count,lanes", [(42, 5, 4096), (42, 10000, 4096), (7, 1000, 64)])
def test_xorshift64_stream_matches_the_scalar_recurrence(seed, count, lanes):
    assert np.array_equal(ics.xorshift64_stream(seed, count, lanes), xorshift64_scalar(seed, count))


def divergence(u, n, l=2.0 * math.pi):
    KX, KY, KZ = ics._k(n, l)
    return np.abs(KX * u[0] + KY * u[1] + KZ * u[2]).max() / max(np.abs(c).max() for c in u) / (n // 2)


def test_von_karman_isotropic_energy_divergence_and_seed():
    n = 16
    u = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=42)
    assert ics.spectral_energy(u, n) == pytest.approx(0.5, rel=1e-12)
    assert divergence(u, n) < 1e-12
    again = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=42)
    assert all(np.array_equal(a, b) for a, b in zip(u, again))
    other = ics.von_karman_isotropic(n, kp=4.0, energy=0.5, seed=43)
    assert not np.allclose(u[0], other[0])


def test_taylor_green_energy():
    assert ics.spectral_energy(ics.taylor_green(16), 16) == pytest.approx(0.125, rel=1e-12)


def test_lamb_oseen_tubes_divergence_free_and_real():
    # real away from the Nyquist planes (with kx[n/2] = -n/2 the curl of a
    # real field is not Hermitian there; the c2r convention drops it)
    n = 32
    u = ics.lamb_oseen_tubes(n)
    assert divergence(u, n) < 1e-12
    keep = np.ones((n, n, n // 2 + 1), dtype=bool)
    keep[n // 2], keep[:, n // 2], keep[:, :, n // 2] = False, False, False
    for c in u:
        back = ics._r2c(ics._c2r(c, n))
        assert np.abs(back - c)[keep].max() <= 1e-12 * np.abs(c).max()


def test_project_control_is_an_idempotent_projection_onto_the_control_space():
    n = 16
    u = ics.von_karman_isotropic(n, seed=5)
    p = ics.project_control(u, n)
    pp = ics.project_control(p, n)
    scale = max(np.abs(c).max() for c in p)
    assert max(np.abs(a - b).max() for a, b in zip(p, pp)) <= 1e-12 * scale
    for c in p:
        assert np.abs(c[n // 2]).max() <= 1e-12 * scale
        assert np.abs(c[:, n // 2]).max() <= 1e-12 * scale
        assert np.abs(c[:, :, n // 2]).max() <= 1e-12 * scale
    assert divergence(p, n) < 1e-12


def test_solenoidal_direction_has_unit_norm():
    n = 16
    v = ics.solenoidal_direction(n, seed=201)
    assert 2.0 * ics.spectral_energy(v, n) == pytest.approx(1.0, rel=1e-12)


class FakeSolver:
    """time advances by dt per step; run() returns one record per step."""

    def __init__(self, dt):
        self.t, self._dt, self.steps = 0.0, dt, 0

    def time(self):
        return self.t

    def dt(self):
        return self._dt

    def run(self, k, every=1):
        recs = []
        for _ in range(k):
            self.t += self._dt
            self.steps += 1
            if self.steps % every == 0:
                recs.append(SimpleNamespace(time=self.t, energy=2.0 * self.t))
        return recs


@pytest.mark.parametrize("dt,t_end", [(0.01, 1.0), (0.003, 0.5), (0.25, 0.1)])
def test_run_to_time_stops_at_the_first_step_reaching_t_end(dt, t_end):
    from vonkarman_gb300.runs import run_to_time

    s = FakeSolver(dt)
    recs = run_to_time(s, t_end)
    assert s.t >= t_end and s.t - dt < t_end          # run.rs:152-155
    assert len(recs) == s.steps


def test_interp_at_is_linear_between_records():
    from vonkarman_gb300.runs import interp_at

    recs = [SimpleNamespace(time=t, energy=3.0 * t + 1.0) for t in (0.0, 0.4, 1.1)]
    assert interp_at(recs, 0.7, "energy") == pytest.approx(3.1)
