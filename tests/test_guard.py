"""The density guard: tests/unit/nan-guard.test.ts and tests/browser/nan-guard.spec.ts
of the reference, restated (host logic on the CPU, the guarded run on the GPU)."""
import math

import numpy as np
import pytest

from pocketwind_gb300 import guard
from pocketwind_gb300._lib import RangeError


@pytest.mark.parametrize("rho", [0.5, 1.0, 1.5])
def test_accepts_physical_density(rho):
    assert not guard.is_unstable_density(rho)


@pytest.mark.parametrize("rho", [math.nan, math.inf, -math.inf, 0.5 - 2 ** -25, 1.5 + 2 ** -23, 0.0, -1.0])
def test_rejects_non_finite_or_out_of_range_density(rho):
    assert guard.is_unstable_density(rho)


def test_reset_comes_before_the_message():
    order = []
    got = []
    msg = guard.reset_unstable_run(600, lambda: order.append("reset"), [lambda m: (order.append("event"), got.append(m))])
    assert order == ["reset", "event"]
    assert msg == guard.Instability(600, "The run went unstable at step 600 and was reset",
                                    "Lower the inflow speed or refine the grid")
    assert got == [msg]


class FakeSolver:
    """Step counting and a scripted guard flag, for the chunking logic."""

    def __init__(self, unstable_after=None):
        self.step_count = 0
        self.calls = []
        self.unstable_after = unstable_after
        self.resets = 0
        self.injected = []

    def step(self, n, macro):
        self.calls.append((self.step_count, n, macro))
        self.step_count += n

    def guard_unstable(self):
        return self.unstable_after is not None and self.step_count > self.unstable_after

    def reset(self):
        self.resets += 1
        self.step_count = 0

    def inject_nan(self):
        self.injected.append(self.step_count)


def test_chunks_stop_at_every_check_and_at_the_injection_step():
    s = FakeSolver()
    g = guard.NanGuard(s, inject_nan=450)
    assert g.advance(1000) is None
    assert [(a, n) for a, n, _ in s.calls] == [(0, 200), (200, 200), (400, 50), (450, 150), (600, 200), (800, 200)]
    assert all(m for _, _, m in s.calls)
    assert s.injected == [450]


def test_injection_at_400_is_caught_at_600_and_resets():
    s = FakeSolver(unstable_after=400)
    g = guard.NanGuard(s, inject_nan=400)
    msg = g.advance(1000)
    assert msg.step == 600 and s.resets == 1 and s.step_count == 0
    assert s.calls[-1][0] + s.calls[-1][1] == 600  # the oversized batch stops at detection


def test_invalid_counts_and_reentry():
    g = guard.NanGuard(FakeSolver())
    for bad in (-1, 1.5, 2 ** 53):
        with pytest.raises(RangeError):
            g.advance(bad)
    g.destroy()
    with pytest.raises(RuntimeError):
        g.advance(1)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_guarded_run_resets_only_an_injected_run(precision):
    """nan-guard.spec.ts:44-177 on the 32^3 domain: an uninjected run passes 1000
    steps; a NaN injected at step 400 is caught at the 600 check, the state is
    reset to equilibrium (finite, step 0)."""
    from pocketwind_gb300 import geometry, solver
    layout = (32, 32, 32)
    cells = 32 ** 3
    geom = np.concatenate([np.zeros(cells, np.uint32), np.full(cells, 0xFFFFFFFF, np.uint32)])
    geom[0] = 4  # the first cell is an equilibrium boundary
    grid = geometry.grid_from_arrays(layout, geom, np.zeros(0, np.uint32))
    params = solver.SolverParams(tau0=0.8, u_in=0.04, precision=precision)
    clean = solver.GpuSolver.create(layout, grid, params)
    assert guard.NanGuard(clean).advance(1000) is None
    assert clean.step_count == 1000
    s = solver.GpuSolver.create(layout, grid, params)
    g = guard.NanGuard(s, inject_nan=400)
    assert g.advance(400) is None
    pops = s.populations().reshape(19, cells)
    assert np.isfinite(pops[:, 0]).all() and np.isnan(pops[:, 1]).any()
    msg = g.advance(600)
    assert msg is not None and msg.step == 600
    assert s.step_count == 0
    assert np.isfinite(s.populations()).all()
    clean.destroy()
    s.destroy()
