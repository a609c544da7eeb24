"""Drag statistics over the force samples a solver run produces.

Host-side binary64 arithmetic, restating the reference's force reporting:

* ``create_drag_stats``: the analysis window of src/forces/drag-stats.ts:161-233
  (window of one flow-through, settling over two, steady when the window's
  relative standard deviation is below 3% and its half-to-half drift below 1%,
  the mean withheld unless five independent batch means support it);
* ``tau_int``, ``batch_length``, ``sem_pct``: drag-stats.ts:78-147;
* ``cd_per_lattice_force``: src/lbm/units.ts:42-45;
* ``flow_through_steps``: src/validation/cases.ts:129-133;
* ``averaged_forces``: the last-two-flow-throughs mean of
  src/validation/runner.ts:234-245.

Samples come from ``GpuSolver.read_force`` (every ``FORCE_EVERY_STEPS`` steps
in the reference's runners, src/lbm/params.ts:12).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence

from ._lib import RangeError

FORCE_EVERY_STEPS = 8
U_LU = 0.05
WINDOW_FLOW_THROUGHS = 1
SETTLING_FLOW_THROUGHS = 2
STEADY_FLUCTUATION_PCT = 3.0
STEADY_DRIFT_PCT = 1.0
MIN_BATCHES = 5
MAX_BATCHES = 16
TOO_FEW_INDEPENDENT_SAMPLES = "too-few-independent-samples"


def _mean(values: Sequence[float]) -> Optional[float]:
    if len(values) == 0:
        return None
    total = 0.0
    for v in values:
        total += v
    return total / len(values)


def _sample_std(values: Sequence[float]) -> float:
    if len(values) < 2:
        return 0.0
    m = _mean(values) or 0.0
    squares = 0.0
    for v in values:
        squares += (v - m) * (v - m)
    return math.sqrt(squares / (len(values) - 1))


def _relative_std_pct(values: Sequence[float]) -> float:
    m = _mean(values)
    if m is None:
        return 0.0
    s = _sample_std(values)
    if m == 0:
        return 0.0 if s == 0 else math.inf
    return 100.0 * s / abs(m)


def _half_drift_pct(values: Sequence[float]) -> float:
    """First half against second half; an odd count leaves the middle in the second half."""
    n = len(values)
    if n < 2:
        return 0.0
    half = n // 2
    first, second, m = _mean(values[:half]), _mean(values[half:]), _mean(values)
    if first is None or second is None or m is None:
        return 0.0
    change = abs(first - second)
    if m == 0:
        return 0.0 if change == 0 else math.inf
    return 100.0 * change / abs(m)


def tau_int(values: Sequence[float], sample_spacing_steps: float = 1) -> float:
    """Integral time in steps: the autocorrelation summed up to its first zero
    crossing, lag zero counting one (drag-stats.ts:78-108)."""
    if not math.isfinite(sample_spacing_steps) or sample_spacing_steps <= 0:
        raise RangeError("Sample spacing must be finite and positive.")
    n = len(values)
    if n < 2:
        return sample_spacing_steps
    m = 0.0
    for v in values:
        m += v
    m /= n
    centred = [v - m for v in values]
    variance = 0.0
    for c in centred:
        variance += c * c
    if variance == 0:
        return sample_spacing_steps
    total = 1.0
    for lag in range(1, n // 2 + 1):
        cov = 0.0
        for i in range(n - lag):
            cov += centred[i] * centred[i + lag]
        if cov <= 0:
            break
        total += cov / variance
    return total * sample_spacing_steps


def batch_length(values: Sequence[float], sample_spacing_steps: float = 1) -> float:
    """Twice the integral time, at least eight force intervals (drag-stats.ts:110-117)."""
    return max(2 * tau_int(values, sample_spacing_steps), 8 * FORCE_EVERY_STEPS)


def sem_pct(values: Sequence[float], sample_spacing_steps: float = 1,
            window_steps: Optional[float] = None) -> Optional[float]:
    """Batch-means standard error of the mean in percent; None when fewer than
    five independent batches fit (drag-stats.ts:119-147)."""
    n = len(values)
    if window_steps is None:
        window_steps = n * sample_spacing_steps
    m = _mean(values)
    if m is None:
        return None
    if not math.isfinite(window_steps) or window_steps <= 0:
        return None
    length = batch_length(values, sample_spacing_steps)
    per_batch = max(1, _round_half_up(length / sample_spacing_steps))
    available = n // per_batch
    batches = min(MAX_BATCHES, math.floor(window_steps / length), available)
    if batches < MIN_BATCHES:
        return None
    start = n - batches * per_batch  # the newest complete batches
    means = []
    for b in range(batches):
        total = 0.0
        lo = start + b * per_batch
        for i in range(lo, lo + per_batch):
            total += values[i]
        means.append(total / per_batch)
    s = _sample_std(means)
    if m == 0:
        return 0.0 if s == 0 else math.inf
    return 100.0 * (s / math.sqrt(batches)) / abs(m)


def _round_half_up(x: float) -> int:
    """JavaScript Math.round: halves go up."""
    return int(math.floor(x + 0.5))


def cd_per_lattice_force(frontal_cells: float, u_lu: float = U_LU) -> float:
    """1 / (0.5 u^2 A): a lattice force times this is Cd (units.ts:42-45)."""
    if not (math.isfinite(frontal_cells) and frontal_cells > 0):
        raise RangeError("Frontal area in cells must be positive and finite.")
    return 1.0 / (0.5 * u_lu * u_lu * frontal_cells)


def flow_through_steps(nx: int, u_lu: float = U_LU) -> int:
    """Steps for the inflow to cross the tunnel once (cases.ts:129-133)."""
    if not isinstance(nx, int) or nx < 1:
        raise RangeError("Grid length must be positive.")
    if not (math.isfinite(u_lu) and u_lu > 0):
        raise RangeError("Inlet speed must be positive.")
    return math.ceil(nx / u_lu)


@dataclass
class DragStatus:
    kind: str  # 'settling' | 'steady' | 'unsteady'
    eta_s: Optional[float] = None
    rel_std_pct: Optional[float] = None
    drift_pct: Optional[float] = None


@dataclass
class DragSummary:
    cd: Optional[float]
    status: DragStatus
    samples: int
    sem_pct: Optional[float] = None
    reason: Optional[str] = None


@dataclass
class DragStats:
    """createDragStats (drag-stats.ts:161-233): push samples, ask for a summary."""
    flow_through_steps: float
    cd_per_force: float = 1.0
    _samples: List[tuple] = field(default_factory=list)

    def __post_init__(self):
        if not (math.isfinite(self.flow_through_steps) and self.flow_through_steps > 0):
            raise RangeError("Flow-through steps must be finite and positive.")
        if not math.isfinite(self.cd_per_force):
            raise RangeError("Cd per unit force must be finite.")
        self._window = WINDOW_FLOW_THROUGHS * self.flow_through_steps
        self._settle = SETTLING_FLOW_THROUGHS * self.flow_through_steps

    def push(self, step: float, fx: float) -> None:
        if not (math.isfinite(step) and math.isfinite(fx)):
            raise RangeError("Drag samples require a finite step and force.")
        if self._samples and step <= self._samples[-1][0]:
            raise RangeError("Drag sample steps must strictly increase.")
        self._samples.append((step, fx))
        while self._samples and self._samples[0][0] <= step - self._settle:
            self._samples.pop(0)

    def _spacing(self) -> float:
        if len(self._samples) < 2:
            return FORCE_EVERY_STEPS
        spacing = (self._samples[-1][0] - self._samples[0][0]) / (len(self._samples) - 1)
        return spacing if math.isfinite(spacing) and spacing > 0 else FORCE_EVERY_STEPS

    def summary(self, steps_per_s: Optional[float]) -> DragSummary:
        elapsed = self._samples[-1][0] if self._samples else 0
        values = [fx for step, fx in self._samples if step > elapsed - self._window]
        all_values = [fx for _, fx in self._samples]
        m = _mean(values)
        sem = sem_pct(all_values, self._spacing(), self._settle)
        cd = m * self.cd_per_force if (m is not None and sem is not None) else None
        reason = TOO_FEW_INDEPENDENT_SAMPLES if sem is None else None
        if elapsed < self._settle:
            eta = None
            if steps_per_s is not None and math.isfinite(steps_per_s) and steps_per_s > 0:
                eta = max(0.0, (self._settle - elapsed) / steps_per_s)
            return DragSummary(cd, DragStatus("settling", eta_s=eta), len(values), sem, reason)
        fluct = _relative_std_pct(values)
        drift = _half_drift_pct(values)
        kind = "steady" if (fluct < STEADY_FLUCTUATION_PCT and drift < STEADY_DRIFT_PCT) else "unsteady"
        return DragSummary(cd, DragStatus(kind, rel_std_pct=fluct, drift_pct=drift), len(values), sem, reason)


def create_drag_stats(flow_through_steps: float, cd_per_force: float = 1.0) -> DragStats:
    return DragStats(flow_through_steps, cd_per_force)


def averaged_forces(samples: Iterable, steps: float, average_steps: float):
    """Mean (fx, fy, fz) of the samples with steps - average_steps < step <= steps
    (inAverageWindow and averagedForces, runner.ts:177-179,234-245; the cases
    average over AVERAGE_THROUGHS = 2 flow-throughs, cases.ts:101,240)."""
    window = [s for s in samples if steps - average_steps < s.step <= steps]
    if not window:
        raise RangeError("No force samples in the averaging window.")
    n = len(window)
    return (sum(s.fx for s in window) / n, sum(s.fy for s in window) / n, sum(s.fz for s in window) / n)
