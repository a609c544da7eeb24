"""ctypes binding of libpocketwind_gb300.so (the C ABI declared in include/pocketwind.h).

The library is the only compute path: every GPU-facing call in this package goes
through it, and a missing library or a CUDA failure raises instead of falling
back to anything else.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

PW_OK, PW_ERR_INVALID, PW_ERR_OOM, PW_ERR_UNSTABLE, PW_ERR_BUSY, PW_ERR_TIMEOUT, PW_ERR_CUDA, PW_ERR_DESTROYED = range(8)


class RangeError(ValueError):
    """Invalid input: the reference throws RangeError for these."""


class AllocationFailure(Exception):
    """Device memory exhausted; the reference returns AllocationFailure (gpu-resources.ts:3-5)."""

    kind = "allocation-failure"


class CudaError(RuntimeError):
    """A CUDA runtime error reported by the library."""


class DomainDesc(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("tau0", C.c_double), ("u_in", C.c_double), ("les", C.c_int), ("op", C.c_int),
                ("walls", C.c_int), ("storage", C.c_int), ("ramp_steps", C.c_uint32), ("strict", C.c_int),
                ("kernel", C.c_int), ("lateral", C.c_int)]


class GridStats(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("solid_cells", C.c_uint32), ("frontal_cells", C.c_uint32), ("watertight", C.c_uint32),
                ("missed_links", C.c_uint32), ("reserved", C.c_uint32), ("blockage", C.c_double),
                ("geometry_len", C.c_uint64), ("boundary_cells", C.c_uint64)]


class ForceSampleC(C.Structure):
    _fields_ = [("step", C.c_uint64), ("fx", C.c_double), ("fy", C.c_double), ("fz", C.c_double)]


_vp, _u32, _u64, _f32, _sz, _int = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_size_t, C.c_int
_PP = C.POINTER(C.c_void_p)

SIGNATURES = {
    "pw_last_error": (C.c_char_p, []),
    "pw_version": (C.c_char_p, []),
    "pw_device_count": (_int, []),
    "pw_voxelize": (_int, [_vp, _u32, _vp, _u32, _u32, _u32, _u32, _int, _PP]),
    "pw_voxelize_opts": (_int, [_vp, _u32, _vp, _u32, _u32, _u32, _u32, _int, _int, _PP]),
    "pw_grid_from_host": (_int, [_u32, _u32, _u32, _vp, _sz, _vp, _sz, _PP]),
    "pw_grid_stats_get": (_int, [_vp, C.POINTER(GridStats)]),
    "pw_grid_read_geometry": (_int, [_vp, _vp, _sz]),
    "pw_grid_read_boundary": (_int, [_vp, _vp, _sz]),
    "pw_grid_destroy": (None, [_vp]),
    "pw_validate_desc": (_int, [C.POINTER(DomainDesc)]),
    "pw_domain_create": (_int, [C.POINTER(DomainDesc), _vp, _PP]),
    "pw_domain_destroy": (None, [_vp]),
    "pw_reset": (_int, [_vp]),
    "pw_step": (_int, [_vp, _u64, _int]),
    "pw_step_count": (_int, [_vp, C.POINTER(C.c_uint64)]),
    "pw_encode_force": (_int, [_vp]),
    "pw_read_force": (_int, [_vp, C.POINTER(ForceSampleC)]),
    "pw_read_macros": (_int, [_vp, _vp]),
    "pw_write_macros": (_int, [_vp, _vp]),
    "pw_read_macros_box": (_int, [_vp, _u32, _u32, _u32, _u32, _u32, _u32, _vp]),
    "pw_read_populations": (_int, [_vp, _vp]),
    "pw_read_populations_raw": (_int, [_vp, _vp]),
    "pw_read_populations_noalloc": (_int, [_vp, _vp]),
    "pw_write_populations": (_int, [_vp, _vp]),
    "pw_write_populations_raw": (_int, [_vp, _vp]),
    "pw_read_totals": (_int, [_vp, _vp]),
    "pw_guard_check": (_int, [_vp, C.POINTER(C.c_int)]),
    "pw_inject_nan": (_int, [_vp]),
    "pw_domain_buffers": (_int, [_vp, _PP, _PP, _PP]),
    "pw_field_vtk_body": (_int, [_vp, C.c_double, _vp, _sz]),
    "pw_checkpoint_size": (_int, [_vp, C.POINTER(_sz)]),
    "pw_checkpoint_save": (_int, [_vp, _vp, _sz]),
    "pw_checkpoint_load": (_int, [_vp, _vp, _sz]),
    "pw_time_steps": (_int, [_vp, _u64, C.POINTER(C.c_float)]),
    "pw_profile_steps": (_int, [_vp, _u64, C.POINTER(C.c_float)]),
    "pw_batch_create": (_int, [C.POINTER(_vp), C.c_uint32, C.POINTER(_vp)]),
    "pw_batch_destroy": (None, [_vp]),
    "pw_batch_step": (_int, [_vp, _u64, _int]),
    "pw_batch_time_steps": (_int, [_vp, _u64, C.POINTER(C.c_float)]),
    "pw_batch_tune": (_int, [_vp, C.c_uint32, C.c_void_p]),
    "pw_batch_reset": (_int, [_vp]),
    "pw_closure_create": (_int, [_u64, C.POINTER(_vp)]),
    "pw_closure_destroy": (None, [_vp]),
    "pw_closure_get_params": (_int, [_vp, _vp]),
    "pw_closure_set_params": (_int, [_vp, _vp]),
    "pw_closure_eval": (_int, [_vp, _vp, C.c_uint32, _vp]),
    "pw_closure_gradients": (_int, [_vp, _vp, _vp, C.c_uint32, _vp, C.POINTER(C.c_float)]),
    "pw_closure_dataset_add": (_int, [_vp, _vp, C.c_double, C.POINTER(_u64)]),
    "pw_closure_dataset_clear": (_int, [_vp]),
    "pw_closure_dataset_reserve": (_int, [_vp, _u64]),
    "pw_closure_dataset_write": (_int, [_vp, _vp, _vp, _u64]),
    "pw_closure_dataset_size": (_int, [_vp, C.POINTER(_u64)]),
    "pw_closure_dataset_read": (_int, [_vp, _u64, _u64, _vp, _vp]),
    "pw_closure_train": (_int, [_vp, C.c_uint32, C.c_uint32, C.c_float, _u64, C.POINTER(C.c_float),
                                C.POINTER(C.c_float)]),
    "pw_closure_attach": (_int, [_vp, _vp]),
    "pw_particles_create": (_int, [_vp, _vp, _u32, _u32, _vp, _vp, _PP]),
    "pw_particles_update": (_int, [_vp, _f32]),
    "pw_particles_read": (_int, [_vp, _vp]),
    "pw_particles_write": (_int, [_vp, _vp]),
    "pw_particles_destroy": (None, [_vp]),
    "pw_plate_create": (_int, [_vp, _u32, _u32, _u32, _vp, _u32, _PP]),
    "pw_plate_advance": (_int, [_vp, _u32, _int, _vp]),
    "pw_plate_read": (_int, [_vp, _vp]),
    "pw_plate_destroy": (None, [_vp]),
    "pw_streaks_create": (_int, [_vp, _u32, _u32, _u32, _vp, _PP]),
    "pw_streaks_advance": (_int, [_vp, _f32, _u32, _int]),
    "pw_streaks_read": (_int, [_vp, _vp, _vp]),
    "pw_streaks_destroy": (None, [_vp]),
}

_lock = threading.Lock()
_lib = None


def load(build_if_stale: bool = True):
    """Load (building first if a source is newer) the shared library."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build() if build_if_stale else _build.LIB
            if not path.exists():
                raise RuntimeError(f"libpocketwind_gb300 is not built ({path}); run __graft_entry__.build()")
            lib = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(rc: int, what: str = "") -> int:
    """Turn a PW_* status into the reference's error behaviour."""
    if rc == PW_OK or rc == PW_ERR_BUSY:
        return rc
    msg = (load().pw_last_error() or b"").decode()
    if what:
        msg = f"{what}: {msg}"
    if rc == PW_ERR_INVALID:
        raise RangeError(msg)
    if rc == PW_ERR_OOM:
        raise AllocationFailure(msg)
    raise CudaError(f"status {rc}: {msg}")


def require_gpu():
    """Raise unless a CUDA device is visible: the library has no CPU path."""
    if load().pw_device_count() < 1:
        raise CudaError("no CUDA device is visible; libpocketwind_gb300 runs on the GPU only")
