"""GpuSolver: the reference's solver interface over libpocketwind_gb300.

Mirrors src/lbm/gpu-solver.ts:135-465 and src/lbm/gpu-force.ts:45-216 (names,
argument meaning and error behaviour):

* ``GpuSolver.create(layout, grid, params)`` returns a solver, or an
  ``AllocationFailure`` (returned, not raised) when device memory runs out; bad
  input raises ``RangeError``.
* ``step(count, write_macro_on_last)`` queues ``count`` fused stream-collide
  steps; ``encode_force()`` / ``read_force()`` sample the mean momentum exchange
  of the two latest states with the reference's single staging slot
  (``read_force`` returns ``'busy'`` when nothing is pending).
* ``macros()``, ``populations()``, ``step_count``, ``reset()``, ``destroy()``.
The WebGPU command encoder disappears: work is queued on the domain's CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Union

import numpy as np

from . import _lib
from ._lib import AllocationFailure, RangeError
from .geometry import VoxelGrid

FORCE_EVERY_STEPS = 8  # src/lbm/params.ts:12
OPERATORS = {"trt": 0, "reg": 1}
WALLS = {"bb": 0, "bouzidi": 1}
PRECISIONS = {"f32": 0, "f16": 1, "bf16": 2}


@dataclass
class SolverParams:
    """SolverParams (gpu-solver.ts:19-30); ``strict`` selects the bit-exact build."""
    tau0: float
    u_in: float
    les: bool = False
    operator: str = "trt"
    walls: str = "bb"
    precision: str = "f32"
    ramp_steps: int = 0
    strict: bool = False
    kernel: str = "auto"  # "auto" or "cell" (one cell per thread), "tile" (x-rows staged in shared memory)
    lateral: str = "periodic"  # or "free-slip": the y and z faces reflect (no counterpart in the reference)


@dataclass
class ForceSample:
    step: int
    fx: float
    fy: float
    fz: float


class GpuSolver:
    def __init__(self, ptr, layout, params: SolverParams):
        self._ptr = ptr
        self.layout = tuple(layout)
        self.params = params
        self.cells = layout[0] * layout[1] * layout[2]
        self.destroyed = False

    # -------------------------------------------------------------- create
    @staticmethod
    def validate(layout, params: SolverParams) -> None:
        """Raise RangeError for parameters that GpuSolver.create would refuse
        before any device work (packSolverParams, gpu-solver.ts:80-116); needs
        the library but no GPU."""
        GpuSolver._desc(layout, params)

    @staticmethod
    def _desc(layout, params: SolverParams):
        ramp = params.ramp_steps
        if not isinstance(ramp, int) or ramp < 0:
            raise RangeError("Ramp steps must be a non-negative safe integer.")
        if params.operator not in OPERATORS or params.walls not in WALLS or params.precision not in PRECISIONS:
            raise RangeError("Unknown operator, wall treatment or precision.")
        if params.lateral not in ("periodic", "free-slip") or params.kernel not in ("auto", "cell", "tile"):
            raise RangeError("Unknown lateral boundary or kernel choice.")
        dims = []
        for v in layout:
            if isinstance(v, bool) or not float(v).is_integer() or not 1 <= v < 2 ** 32:
                raise RangeError("Grid dimensions must be positive safe integers.")
            dims.append(int(v))
        d = _lib.DomainDesc(*dims, float(params.tau0), float(params.u_in), int(bool(params.les)),
                            OPERATORS[params.operator], WALLS[params.walls], PRECISIONS[params.precision],
                            ramp, int(bool(params.strict)), {"auto": 0, "cell": 1, "tile": 2}[params.kernel],
                            {"periodic": 0, "free-slip": 1}[params.lateral])
        _lib.check(_lib.load().pw_validate_desc(C.byref(d)), "GpuSolver.create")
        return d

    @staticmethod
    def create(layout, grid: VoxelGrid, params: SolverParams) -> Union["GpuSolver", AllocationFailure]:
        d = GpuSolver._desc(layout, params)
        nx, ny, nz = d.nx, d.ny, d.nz
        if (nx, ny, nz) != (grid.nx, grid.ny, grid.nz):
            raise RangeError("Geometry must match the solver layout and contain flags and q offsets.")
        L = _lib.load()
        _lib.require_gpu()
        out = C.c_void_p()
        rc = L.pw_domain_create(C.byref(d), grid._handle.ptr, C.byref(out))
        if rc == _lib.PW_ERR_OOM:
            return AllocationFailure((L.pw_last_error() or b"").decode())
        _lib.check(rc, "GpuSolver.create")
        return GpuSolver(out.value, (nx, ny, nz), params)

    # -------------------------------------------------------------- lifecycle
    def _live(self):
        if self.destroyed:
            raise RuntimeError("The solver has been destroyed.")
        return self._ptr

    def destroy(self) -> None:
        if self.destroyed:
            return
        _lib.load().pw_domain_destroy(self._ptr)
        self._ptr = None
        self.destroyed = True

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def reset(self) -> None:
        _lib.check(_lib.load().pw_reset(self._live()), "reset")

    # -------------------------------------------------------------- stepping
    def step(self, count: int, write_macro_on_last: bool = False) -> None:
        if not isinstance(count, (int, np.integer)) or count < 0:
            raise RangeError("Step count must be a non-negative safe integer.")
        _lib.check(_lib.load().pw_step(self._live(), int(count), int(bool(write_macro_on_last))), "step")

    @property
    def step_count(self) -> int:
        v = C.c_uint64()
        _lib.check(_lib.load().pw_step_count(self._live(), C.byref(v)))
        return v.value

    def time_steps(self, count: int) -> float:
        """Device milliseconds of ``count`` steps, timed with CUDA events on the solver's stream."""
        ms = C.c_float()
        _lib.check(_lib.load().pw_time_steps(self._live(), int(count), C.byref(ms)), "time_steps")
        return ms.value

    def profile_steps(self, count: int) -> tuple:
        """Summed device milliseconds of the plain-cell, seam-row and edge-cell
        kernels over ``count`` steps (CUDA events around each launch)."""
        ms = (C.c_float * 3)()
        _lib.check(_lib.load().pw_profile_steps(self._live(), int(count), ms), "profile_steps")
        return tuple(ms)

    # -------------------------------------------------------------- force
    def encode_force(self) -> None:
        _lib.check(_lib.load().pw_encode_force(self._live()), "encode_force")

    def read_force(self) -> Union[ForceSample, str]:
        s = _lib.ForceSampleC()
        rc = _lib.load().pw_read_force(self._live(), C.byref(s))
        if rc == _lib.PW_ERR_BUSY:
            return "busy"
        _lib.check(rc, "read_force")
        return ForceSample(s.step, s.fx, s.fy, s.fz)

    # -------------------------------------------------------------- fields
    def macros(self, out: np.ndarray = None) -> np.ndarray:
        """(rho, ux, uy, uz) per cell (macroBuffer, docs/numerics.md:147-155), into `out` when
        given: a C-contiguous float32 array of shape (cells, 4) that the caller keeps from
        one readout to the next."""
        if out is None:
            out = np.empty((self.cells, 4), np.float32)
        elif (not isinstance(out, np.ndarray) or out.dtype != np.float32 or out.shape != (self.cells, 4)
              or not out.flags.c_contiguous or not out.flags.writeable):
            raise RangeError("out must be a writeable C-contiguous float32 array of shape (cells, 4).")
        _lib.check(_lib.load().pw_read_macros(self._live(), out.ctypes.data_as(C.c_void_p)), "macros")
        return out

    def macros_box(self, origin, size) -> np.ndarray:
        """Macros (rho, ux, uy, uz) of a box of cells, shape (wz, wy, wx, 4)."""
        x0, y0, z0 = (int(v) for v in origin)
        wx, wy, wz = (int(v) for v in size)
        out = np.empty((wz, wy, wx, 4), np.float32)
        _lib.check(_lib.load().pw_read_macros_box(self._live(), x0, y0, z0, wx, wy, wz,
                                                  out.ctypes.data_as(C.c_void_p)), "macros_box")
        return out

    def write_macros(self, macros: np.ndarray) -> None:
        a = np.ascontiguousarray(macros, np.float32).reshape(-1)
        if a.size != 4 * self.cells:
            raise RangeError("Macros must hold 4 values per cell.")
        _lib.check(_lib.load().pw_write_macros(self._live(), a.ctypes.data_as(C.c_void_p)), "write_macros")

    def populations(self) -> np.ndarray:
        out = np.empty(19 * self.cells, np.float32)
        _lib.check(_lib.load().pw_read_populations(self._live(), out.ctypes.data_as(C.c_void_p)), "populations")
        return out

    def populations_raw(self) -> np.ndarray:
        dt = np.float32 if self.params.precision == "f32" else np.uint16
        out = np.empty(19 * self.cells, dt)
        _lib.check(_lib.load().pw_read_populations_raw(self._live(), out.ctypes.data_as(C.c_void_p)), "populations")
        return out

    def write_populations(self, g: np.ndarray) -> None:
        a = np.ascontiguousarray(g, np.float32).reshape(-1)
        if a.size != 19 * self.cells:
            raise RangeError("Populations must hold 19 values per cell.")
        _lib.check(_lib.load().pw_write_populations(self._live(), a.ctypes.data_as(C.c_void_p)), "write")

    def write_populations_raw(self, raw: np.ndarray) -> None:
        dt = np.float32 if self.params.precision == "f32" else np.uint16
        a = np.ascontiguousarray(raw, dt).reshape(-1)
        if a.size != 19 * self.cells:
            raise RangeError("Populations must hold 19 values per cell.")
        _lib.check(_lib.load().pw_write_populations_raw(self._live(), a.ctypes.data_as(C.c_void_p)), "write")

    def totals(self) -> np.ndarray:
        """FP64 (mass deviation, momentum x, y, z) of the latest state."""
        out = np.zeros(4, np.float64)
        _lib.check(_lib.load().pw_read_totals(self._live(), out.ctypes.data_as(C.c_void_p)), "totals")
        return out

    def guard_unstable(self) -> bool:
        v = C.c_int()
        _lib.check(_lib.load().pw_guard_check(self._live(), C.byref(v)), "guard")
        return bool(v.value)

    def inject_nan(self) -> None:
        _lib.check(_lib.load().pw_inject_nan(self._live()), "inject_nan")

    # -------------------------------------------------------------- state export
    def field_vtk_body(self, velocity_scale: float) -> bytes:
        """The VTK bytes after writeVtk's header for the macros as last written,
        velocity scaled by ``velocity_scale`` (pw_field_vtk_body)."""
        n = 16 * self.cells + 25
        out = np.empty(n, np.uint8)
        _lib.check(_lib.load().pw_field_vtk_body(self._live(), float(velocity_scale),
                                                 out.ctypes.data_as(C.c_void_p), n), "field_vtk_body")
        return out.tobytes()

    def save_checkpoint(self) -> bytes:
        """The solver state as a self-checking blob (pw_checkpoint_save)."""
        n = C.c_size_t()
        L = _lib.load()
        _lib.check(L.pw_checkpoint_size(self._live(), C.byref(n)), "checkpoint")
        out = np.empty(n.value, np.uint8)
        _lib.check(L.pw_checkpoint_save(self._live(), out.ctypes.data_as(C.c_void_p), n.value), "checkpoint")
        return out.tobytes()

    def load_checkpoint(self, blob: bytes) -> None:
        """Restore a state saved by a solver of the same layout and parameters."""
        a = np.frombuffer(blob, np.uint8)
        _lib.check(_lib.load().pw_checkpoint_load(self._live(), a.ctypes.data_as(C.c_void_p), a.size),
                   "load_checkpoint")

    def buffers(self):
        m, f, s = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _lib.check(_lib.load().pw_domain_buffers(self._live(), C.byref(m), C.byref(f), C.byref(s)))
        return m.value, f.value, s.value
