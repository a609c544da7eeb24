"""The C ABI boundary on the CPU: the library builds and loads, exports every
entry point include/pocketwind.h declares, and refuses to compute without a GPU
(there is no host fallback)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "pocketwind.h").read_text()
    return sorted(set(re.findall(r"^PW_API\s+[^(]*?\b(pw_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_symbols()
    for required in ("pw_domain_create", "pw_step", "pw_encode_force", "pw_read_force", "pw_voxelize",
                     "pw_read_macros", "pw_streaks_advance", "pw_particles_update", "pw_plate_advance"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from pocketwind_gb300 import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


def test_version_and_errors_without_compute():
    from pocketwind_gb300 import _lib
    lib = _lib.load()
    assert b"sm_103a" in lib.pw_version()
    out = C.c_void_p()
    rc = lib.pw_voxelize(None, 0, None, 0, 1, 8, 8, 0, C.byref(out))
    assert rc == _lib.PW_ERR_INVALID and b"at least two" in lib.pw_last_error()
    assert lib.pw_step(None, 1, 0) == _lib.PW_ERR_INVALID
    lib.pw_domain_destroy(None)
    lib.pw_grid_destroy(None)


def test_no_gpu_means_loud_failure():
    from pocketwind_gb300 import _lib
    if _lib.load().pw_device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(_lib.CudaError):
        _lib.require_gpu()
