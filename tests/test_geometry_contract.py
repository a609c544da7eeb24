"""The packed-geometry checks that run on the host before any device work,
restating tests/unit/geometry-contract.test.ts (validateGeometry,
src/lbm/geometry-contract.ts:39-66): cell kinds, q offsets in packing order
and the geometry length.  The pull-mask consistency checks run on the GPU
(tests/test_gpu_solver.py); here a grid that passes the host checks reaches the
device allocation, which fails without a GPU (CudaError, not RangeError)."""
import numpy as np
import pytest

from pocketwind_gb300 import geometry as G
from pocketwind_gb300._lib import CudaError, RangeError
from tests.shapes import FLOOR, NO_Q, SOLID, SUPPORT

LAYOUT = (3, 1, 1)
# with singleton periodic y/z axes, five pulls in each x direction hit the wall
POSITIVE_X = sum(1 << (3 + i) for i in (1, 7, 9, 13, 15))
NEGATIVE_X = sum(1 << (3 + i) for i in (2, 8, 10, 14, 16))


def wall_grid(kind, with_fractions=False):
    geometry = np.zeros(16 if with_fractions else 6, np.uint32)
    geometry[:6] = [kind, POSITIVE_X, NEGATIVE_X, NO_Q, NO_Q, NO_Q]
    if with_fractions:
        geometry[4:6] = [0, 5]
        geometry[6:] = np.full(10, 0.5, np.float32).view(np.uint32)
    return geometry, np.array([1, 2], np.uint32)


def accepted_on_the_host(geometry, boundary):
    try:
        G.grid_from_arrays(LAYOUT, geometry, boundary)
    except CudaError:
        pass  # past the checks, at the device allocation (no GPU here)


@pytest.mark.parametrize("kind", [SOLID, SUPPORT, FLOOR])
@pytest.mark.parametrize("with_fractions", [False, True])
def test_accepts_complete_periodic_masks(kind, with_fractions):
    accepted_on_the_host(*wall_grid(kind, with_fractions))


@pytest.mark.parametrize("offset", [0, 4, 6, NO_Q])
def test_rejects_an_inconsistent_q_offset(offset):
    geometry, boundary = wall_grid(SOLID, True)
    geometry[5] = offset
    with pytest.raises(RangeError, match="(?i)geometry"):
        G.grid_from_arrays(LAYOUT, geometry, boundary)


@pytest.mark.parametrize("change", [-1, 1])
def test_rejects_fraction_storage_of_the_wrong_length(change):
    geometry, boundary = wall_grid(SOLID, True)
    resized = np.zeros(geometry.size + change, np.uint32)
    resized[:min(geometry.size, resized.size)] = geometry[:resized.size]
    with pytest.raises(RangeError, match="(?i)geometry length"):
        G.grid_from_arrays(LAYOUT, resized, boundary)


def test_rejects_unknown_kinds_and_boundary_cells_without_links():
    geometry, boundary = wall_grid(SOLID)
    bad = geometry.copy()
    bad[0] = 5  # no cell kind above EQ
    with pytest.raises(RangeError, match="(?i)kind"):
        G.grid_from_arrays(LAYOUT, bad, boundary)
    with pytest.raises(RangeError, match="(?i)boundary"):
        G.grid_from_arrays(LAYOUT, geometry, np.array([0], np.uint32))  # the wall cell itself
    with pytest.raises(RangeError, match="(?i)boundary"):
        G.grid_from_arrays(LAYOUT, geometry, np.array([3], np.uint32))  # past the grid
