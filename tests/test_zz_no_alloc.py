"""The allocation-free population readout, checked against the allocating one.

pw_read_populations_noalloc serves callers that cannot call cudaMalloc when they
read a domain back -- a GPU whose memory is already taken by its domains, or a
host that budgets device memory once up front -- by converting the state
through a fixed 4 MiB array in the library's device image instead of a
19 x cells x 4-byte buffer.  These tests call it through the C ABI and compare
it with pw_read_populations (the same decoded values, so the comparison is
exact), on two calls in a row, on both step parities of the in-place layout,
across several slabs per direction, and check that an oversized plane is
rejected.  It also reads the device's free memory before the first readout and
after the second: creating the domain has already loaded the readout's code and
array (CUDA loads them lazily, and loading takes memory), so the readout itself
takes nothing.  This file runs last so that a failure here leaves every other
test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    fn = lib.pw_read_populations_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p]
    return fn


def _free_device_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _solver(layout, precision):
    from pocketwind_gb300 import geometry, meshes, solver
    nx, ny, nz = layout
    grid = geometry.voxelize(meshes.icosphere((nx / 4, ny / 2, nz / 2), 6, 3), None, layout, False)
    s = solver.GpuSolver.create(layout, grid, solver.SolverParams(tau0=0.6, u_in=0.05, precision=precision))
    assert not isinstance(s, Exception)
    return s


@pytest.mark.parametrize("precision", ["f16", "f32"])
def test_noalloc_readout_matches_allocating_readout(precision):
    from pocketwind_gb300 import _lib
    lib = _lib.load()
    read = _noalloc(lib)
    # 512 x 256 planes: 512 KiB per direction plane, 8 planes per slab, 3 slabs per direction
    s = _solver((512, 256, 24), precision)
    s.step(5)  # odd layout
    expected = s.populations()  # allocates the domain's readout buffer on first use
    free_before = _free_device_bytes()
    for _ in range(2):
        out = np.full(19 * s.cells, np.nan, np.float32)
        rc = read(s._ptr, out.ctypes.data_as(C.c_void_p))
        assert rc == _lib.PW_OK, lib.pw_last_error()
        np.testing.assert_array_equal(out, expected)
    assert _free_device_bytes() == free_before  # nothing was allocated or loaded
    s.step(3)  # even layout
    expected = s.populations()
    out = np.full(19 * s.cells, np.nan, np.float32)
    assert read(s._ptr, out.ctypes.data_as(C.c_void_p)) == _lib.PW_OK
    np.testing.assert_array_equal(out, expected)
    s.destroy()


def test_noalloc_readout_rejects_planes_beyond_its_array():
    from pocketwind_gb300 import _lib, geometry, solver
    lib = _lib.load()
    read = _noalloc(lib)
    layout = (2048, 520, 2)  # 1,064,960 cells per plane: 4.26 MB > 4 MiB
    cells = 2048 * 520 * 2
    geom = np.concatenate([np.zeros(cells, np.uint32), np.full(cells, 0xFFFFFFFF, np.uint32)])
    grid = geometry.grid_from_arrays(layout, geom, np.zeros(0, np.uint32))
    s = solver.GpuSolver.create(layout, grid, solver.SolverParams(tau0=0.6, u_in=0.05))
    out = np.zeros(19 * cells, np.float32)
    rc = read(s._ptr, out.ctypes.data_as(C.c_void_p))
    assert rc == _lib.PW_ERR_INVALID
    assert b"at most 1048576" in lib.pw_last_error()
    s.destroy()
