"""The learned subgrid closure (the C ABI's pw_closure_*).

A 9 -> 32 -> 32 -> 1 network whose output c scales the Smagorinsky eddy
viscosity of plain LES cells by max(0, 1 + c); the untrained network (zero
output layer) is plain Smagorinsky.  Training data come from the solver's own
fine-grid runs, box-filtered onto the 2x coarser grid; training (forward,
backward, Adam) and the inference fused into the step kernel run on the GPU.
No counterpart in the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

N_PARAMS = 1409
N_IN = 9


def _f32(a, n=None):
    a = np.ascontiguousarray(a, np.float32)
    if n is not None and a.size != n:
        raise _lib.RangeError(f"expected {n} values, got {a.size}")
    return a


class Closure:
    def __init__(self, seed: int = 1):
        out = C.c_void_p()
        _lib.check(_lib.load().pw_closure_create(int(seed), C.byref(out)), "Closure")
        self._ptr = out.value

    def _live(self):
        if not self._ptr:
            raise RuntimeError("The closure has been destroyed.")
        return self._ptr

    @property
    def params(self) -> np.ndarray:
        out = np.empty(N_PARAMS, np.float32)
        _lib.check(_lib.load().pw_closure_get_params(self._live(), out.ctypes.data_as(C.c_void_p)), "params")
        return out

    @params.setter
    def params(self, w) -> None:
        w = _f32(w, N_PARAMS)
        _lib.check(_lib.load().pw_closure_set_params(self._live(), w.ctypes.data_as(C.c_void_p)), "params")

    def eval(self, x) -> np.ndarray:
        x = _f32(x).reshape(-1, N_IN)
        out = np.empty(len(x), np.float32)
        _lib.check(_lib.load().pw_closure_eval(self._live(), x.ctypes.data_as(C.c_void_p), len(x),
                                               out.ctypes.data_as(C.c_void_p)), "eval")
        return out

    def gradients(self, x, y):
        x = _f32(x).reshape(-1, N_IN)
        y = _f32(y, len(x))
        g = np.empty(N_PARAMS, np.float32)
        loss = C.c_float()
        _lib.check(_lib.load().pw_closure_gradients(self._live(), x.ctypes.data_as(C.c_void_p),
                                                    y.ctypes.data_as(C.c_void_p), len(x),
                                                    g.ctypes.data_as(C.c_void_p), C.byref(loss)), "gradients")
        return loss.value, g

    # ------------------------------------------------------------ dataset
    def add_samples(self, fine_solver, nu0_coarse: float) -> int:
        n = C.c_uint64()
        _lib.check(_lib.load().pw_closure_dataset_add(self._live(), fine_solver._live(), float(nu0_coarse),
                                                      C.byref(n)), "add_samples")
        return n.value

    def set_dataset(self, x, y) -> None:
        x = _f32(x).reshape(-1, N_IN)
        y = _f32(y, len(x))
        _lib.check(_lib.load().pw_closure_dataset_write(self._live(), x.ctypes.data_as(C.c_void_p),
                                                        y.ctypes.data_as(C.c_void_p), len(x)), "set_dataset")

    @property
    def dataset_size(self) -> int:
        n = C.c_uint64()
        _lib.check(_lib.load().pw_closure_dataset_size(self._live(), C.byref(n)), "dataset_size")
        return n.value

    def dataset(self, first: int = 0, count=None):
        count = self.dataset_size - first if count is None else count
        x = np.empty((count, N_IN), np.float32)
        y = np.empty(count, np.float32)
        _lib.check(_lib.load().pw_closure_dataset_read(self._live(), int(first), int(count),
                                                       x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p)),
                   "dataset")
        return x, y

    def clear_dataset(self) -> None:
        _lib.check(_lib.load().pw_closure_dataset_clear(self._live()), "clear_dataset")

    # ------------------------------------------------------------ training
    def train(self, steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 1):
        first, last = C.c_float(), C.c_float()
        _lib.check(_lib.load().pw_closure_train(self._live(), int(steps), int(batch), float(lr), int(seed),
                                                C.byref(first), C.byref(last)), "train")
        return first.value, last.value

    def attach(self, solver) -> None:
        _lib.check(_lib.load().pw_closure_attach(solver._live(), self._live()), "attach")
        solver._closure = self

    @staticmethod
    def detach(solver) -> None:
        _lib.check(_lib.load().pw_closure_attach(solver._live(), None), "detach")
        solver._closure = None

    def destroy(self) -> None:
        if self._ptr:
            _lib.load().pw_closure_destroy(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
