"""The density guard around a solver run: NanGuard of src/lbm/nan-guard.ts:97-196.

Every ``NAN_GUARD_INTERVAL`` steps the last step of the chunk writes macros and
the step kernel raises the domain's status flag if any cell's density is not
finite or lies outside [0.5, 1.5] (the reference scans the macro buffer with
nan_guard.wgsl after that step; the fused flag sees the same values).  A
tripped check resets the solver to its start state, then reports the
instability, and the rest of the batch is not run.  ``inject_nan`` (the
reference's runner parameter) plants a NaN after the chunk that reaches that
step.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

from ._lib import RangeError

NAN_GUARD_INTERVAL = 200
_MAX_SAFE = 2 ** 53 - 1

# The instability event's text: what happened, and what a caller can change
# (the inflow speed, or the grid resolution, which raises tau0 at a given Re).
RUN_UNSTABLE_WHAT = "The run went unstable at step N and was reset"
RUN_UNSTABLE_NEXT = "Lower the inflow speed or refine the grid"


def is_unstable_density(rho: float) -> bool:
    """nan-guard.ts:39: not finite or outside [0.5, 1.5], both endpoints allowed."""
    return not math.isfinite(rho) or rho < 0.5 or rho > 1.5


@dataclass(frozen=True)
class Instability:
    step: int
    what: str
    next: str


def reset_unstable_run(step: int, reset, listeners=()) -> Instability:
    """resetUnstableRun (nan-guard.ts:58-72): reset first, then publish."""
    reset()
    message = Instability(step, RUN_UNSTABLE_WHAT.replace("step N", f"step {step}"), RUN_UNSTABLE_NEXT)
    for listener in listeners:
        listener(message)
    return message


class NanGuard:
    """Guarded stepping of one GpuSolver."""

    def __init__(self, solver, inject_nan: Optional[int] = None):
        self.solver = solver
        self.inject_nan = inject_nan
        self.listeners = []
        self._advancing = False
        self._destroyed = False

    def add_listener(self, fn) -> None:
        self.listeners.append(fn)

    def advance(self, count: int) -> Optional[Instability]:
        if self._destroyed:
            raise RuntimeError("The density guard has been destroyed.")
        if self._advancing:
            raise RuntimeError("Await the previous advance before stepping again.")
        start = self.solver.step_count
        if not isinstance(count, int) or count < 0 or start + count > _MAX_SAFE:
            raise RangeError("Step count must be a non-negative safe integer.")
        self._advancing = True
        try:
            remaining = count
            while remaining > 0:
                now = self.solver.step_count
                until_check = NAN_GUARD_INTERVAL - now % NAN_GUARD_INTERVAL
                inj = self.inject_nan
                until_inj = inj - now if (isinstance(inj, int) and inj > now) else math.inf
                steps = int(min(remaining, until_check, until_inj))
                self.solver.step(steps, True)
                remaining -= steps
                if self.solver.step_count % NAN_GUARD_INTERVAL == 0 and self.solver.guard_unstable():
                    return reset_unstable_run(self.solver.step_count, self.solver.reset, self.listeners)
                if isinstance(inj, int) and self.solver.step_count == inj:
                    self.solver.inject_nan()
            return None
        finally:
            self._advancing = False

    def destroy(self) -> None:
        if self._advancing:
            raise RuntimeError("Await advance before destroying the density guard.")
        self._destroyed = True
