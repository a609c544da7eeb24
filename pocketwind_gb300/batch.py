"""Many independent domains stepped together (the C ABI's pw_batch_*).

No counterpart in the reference, which runs one solver at a time
(src/app/solver-slot.ts).  Members are ``GpuSolver`` domains of the fast build
(``strict=False``, kernel "auto"/"cell") sharing storage, collision operator and
LES, with equal step counts and no inlet ramp in progress.  Each batch step is
two persistent launches over all members' work, side by side on two streams:
one over every member's plain cells, one over their seam rows and edge cells
(each kernel carries only its own code path and registers; one launch that
carried every path's registers measured 21% slower).  Steps are replayed from
captured CUDA graphs; ``tune`` times the candidate launch shapes and keeps the
fastest.  The members keep their own force, macro and readout calls.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

from . import _lib


class _Tuning(C.Structure):
    _fields_ = [("blocks", C.c_uint32), ("rows_per_item", C.c_uint32), ("ms_per_step", C.c_float),
                ("candidates", C.c_uint32)]


@dataclass(frozen=True)
class Tuning:
    blocks: int
    rows_per_item: int
    ms_per_step: float
    candidates: int


class Batch:
    def __init__(self, members: Sequence):
        self.members = list(members)
        L = _lib.load()
        arr = (C.c_void_p * len(self.members))(*[m._live() for m in self.members])
        out = C.c_void_p()
        _lib.check(L.pw_batch_create(arr, len(self.members), C.byref(out)), "Batch")
        self._ptr = out.value

    def _live(self):
        if not self._ptr:
            raise RuntimeError("The batch has been destroyed.")
        for m in self.members:
            m._live()
        return self._ptr

    def step(self, count: int, write_macro_on_last: bool = False) -> None:
        _lib.check(_lib.load().pw_batch_step(self._live(), int(count), int(bool(write_macro_on_last))), "Batch.step")

    def time_steps(self, count: int) -> float:
        ms = C.c_float()
        _lib.check(_lib.load().pw_batch_time_steps(self._live(), int(count), C.byref(ms)), "Batch.time_steps")
        return ms.value

    def tune(self, trial_steps: int = 8) -> Tuning:
        t = _Tuning()
        _lib.check(_lib.load().pw_batch_tune(self._live(), int(trial_steps), C.cast(C.pointer(t), C.c_void_p)),
                   "Batch.tune")
        return Tuning(t.blocks, t.rows_per_item, t.ms_per_step, t.candidates)

    def reset(self) -> None:
        _lib.check(_lib.load().pw_batch_reset(self._live()), "Batch.reset")

    @property
    def cells(self) -> int:
        return sum(m.cells for m in self.members)

    def destroy(self) -> None:
        if self._ptr:
            _lib.load().pw_batch_destroy(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
