"""Drag statistics: tests/unit/forces/drag-stats.test.ts of the reference, restated.

The seeded series use the mulberry32 generator and the Box-Muller normal of the
reference's test (its published algorithm, written here in Python with 32-bit
wrap-around), so the seeded estimates are the same draws.
"""
import math

import pytest

from pocketwind_gb300 import forces
from pocketwind_gb300._lib import RangeError

FLOW_THROUGH = 100


def mulberry32(seed):
    state = seed & 0xFFFFFFFF

    def imul(a, b):
        return (a * b) & 0xFFFFFFFF

    def nxt():
        nonlocal state
        state = (state + 0x6D2B79F5) & 0xFFFFFFFF
        t = state
        t = imul(t ^ (t >> 15), t | 1)
        t ^= (t + imul(t ^ (t >> 7), t | 61)) & 0xFFFFFFFF
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296

    return nxt


def standard_normal(rand):
    return math.sqrt(-2 * math.log(1 - rand())) * math.cos(2 * math.pi * rand())


def naive_sem_pct(values):
    m = sum(values) / len(values)
    var = sum((v - m) ** 2 for v in values) / (len(values) - 1)
    return 100 * math.sqrt(var / len(values)) / abs(m)


def constant_series(fx, last_step):
    stats = forces.create_drag_stats(400)
    for step in range(0, last_step + 1, 10):
        stats.push(step, fx)
    return stats


def test_constant_force_is_steady_without_fluctuation_or_drift():
    s = constant_series(12, 2400).summary(None)
    assert (s.status.kind, s.status.rel_std_pct, s.status.drift_pct) == ("steady", 0, 0)
    assert s.cd == 12
    assert s.samples == 40
    assert s.sem_pct == 0


def test_ten_percent_sine_is_unsteady():
    stats = forces.create_drag_stats(FLOW_THROUGH)
    for step in range(0, 1001):
        stats.push(step, 10 + math.sin(2 * math.pi * step / 200))
    assert stats.summary(None).status.kind == "unsteady"


def test_settling_during_a_ramp_then_steady():
    stats = forces.create_drag_stats(FLOW_THROUGH)
    for step in range(0, 101, 10):
        stats.push(step, step / 20)
    st = stats.summary(None).status
    assert (st.kind, st.eta_s) == ("settling", None)
    st = stats.summary(50).status
    assert (st.kind, st.eta_s) == ("settling", 2)
    for step in range(110, 1201, 10):
        stats.push(step, 10)
    assert stats.summary(None).status.kind == "steady"


def test_one_and_a_half_percent_drift_is_unsteady():
    stats = forces.create_drag_stats(800)
    for step in range(0, 1601, 10):
        stats.push(step, 10 * (1 + 0.0000375 * (step - 800)))
    s = stats.summary(None)
    assert s.status.kind == "unsteady"
    assert s.status.drift_pct > 1
    assert s.status.rel_std_pct < 1


def test_sparse_and_dense_samples_give_the_same_mean():
    dense, sparse = forces.create_drag_stats(1000), forces.create_drag_stats(1000)
    for step in range(0, 3151):
        dense.push(step, 10 + math.sin(2 * math.pi * step / 50))
    for step in range(0, 3151, 50):
        sparse.push(step, 10 + math.sin(2 * math.pi * step / 50))
    assert abs(dense.summary(None).cd - sparse.summary(None).cd) < 1e-12


def test_white_noise_standard_error_from_batch_means():
    rand = mulberry32(42)
    values = [1 + 0.02 * standard_normal(rand) for _ in range(512)]
    expected = 2 / math.sqrt(512)
    est = forces.sem_pct(values)
    assert est is not None
    assert abs(est / expected - 1) < 0.25


def test_autocorrelated_samples_inflate_the_standard_error():
    rand = mulberry32(7)
    innovation = 0.02 * math.sqrt(1 - 0.9 * 0.9)
    state = 0.0
    for _ in range(200):
        state = 0.9 * state + innovation * standard_normal(rand)
    values = []
    for _ in range(512):
        state = 0.9 * state + innovation * standard_normal(rand)
        values.append(1 + state)
    assert forces.sem_pct(values) >= 2 * naive_sem_pct(values)


def test_too_few_independent_samples_withholds_cd():
    stats = forces.create_drag_stats(250)
    for step in range(0, 2001):
        stats.push(step, math.sin(2 * math.pi * step / 1000))
    s = stats.summary(None)
    assert s.cd is None and s.sem_pct is None
    assert s.reason == forces.TOO_FEW_INDEPENDENT_SAMPLES


def test_sine_batches_cover_a_third_of_its_period():
    period = 2000
    values = [math.sin(2 * math.pi * step / period) for step in range(10241)]
    assert forces.batch_length(values) >= 0.3 * period


def test_white_noise_integral_time_is_one_interval():
    assert forces.tau_int([1, -1, 1, -1, 1, -1, 1, -1], 8) == 8


def test_invalid_configuration_and_out_of_order_samples():
    with pytest.raises(RangeError):
        forces.create_drag_stats(0)
    with pytest.raises(RangeError):
        forces.create_drag_stats(FLOW_THROUGH, float("nan"))
    with pytest.raises(RangeError):
        forces.tau_int([1, 2, 3], 0)
    stats = forces.create_drag_stats(FLOW_THROUGH)
    stats.push(10, 1)
    with pytest.raises(RangeError):
        stats.push(10, 2)
    with pytest.raises(RangeError):
        stats.push(11, float("nan"))


def test_cd_per_lattice_force_and_flow_through():
    """units.ts:42-45 and cases.ts:129-133."""
    assert forces.cd_per_lattice_force(100) == 1 / (0.5 * 0.05 * 0.05 * 100)
    assert forces.flow_through_steps(96) == 1920
    assert forces.flow_through_steps(97) == 1940
    with pytest.raises(RangeError):
        forces.cd_per_lattice_force(0)
    with pytest.raises(RangeError):
        forces.flow_through_steps(0)


def test_averaged_forces_window():
    """runner.ts:177-179: steps - average < step <= steps."""
    class S:
        def __init__(self, step, fx):
            self.step, self.fx, self.fy, self.fz = step, fx, 2 * fx, 3 * fx
    samples = [S(k, float(k)) for k in range(0, 101, 10)]
    fx, fy, fz = forces.averaged_forces(samples, 100, 40)
    assert fx == (70 + 80 + 90 + 100) / 4 and fy == 2 * fx and fz == 3 * fx
    with pytest.raises(RangeError):
        forces.averaged_forces(samples, 200, 50)
