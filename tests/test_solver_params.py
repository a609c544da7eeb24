"""The solver's parameter checks on the CPU, restating the reference's
tests/unit/gpu-solver.test.ts:34-62 (packSolverParams throws RangeError before
any device work): the same grid dimensions, relaxation times and inlet speeds
are refused through pw_validate_desc, which GpuSolver.create runs first."""
import math

import pytest

from pocketwind_gb300.solver import GpuSolver, SolverParams
from pocketwind_gb300._lib import RangeError

LAYOUT = (32, 16, 8)


def params(**kw):
    base = dict(tau0=0.8, u_in=0.04, les=False)
    base.update(kw)
    return SolverParams(**base)


def test_valid_parameters_pass():
    GpuSolver.validate(LAYOUT, params())
    GpuSolver.validate(LAYOUT, params(les=True, operator="reg", precision="f16", walls="bouzidi"))


@pytest.mark.parametrize("nx", [0, -1, 1.5, math.nan, math.inf])
def test_rejects_invalid_grid_dimension(nx):
    with pytest.raises(RangeError):
        GpuSolver.validate((nx, 16, 8), params())


@pytest.mark.parametrize("tau0", [0.5, 0.0, math.nan, math.inf, 1e100, 0.5 + 2.0 ** -52, 0.5 + 2.0 ** -26])
def test_rejects_invalid_relaxation_time(tau0):
    with pytest.raises(RangeError):
        GpuSolver.validate(LAYOUT, params(tau0=tau0))


@pytest.mark.parametrize("u_in", [1e100, -1e100, math.inf, -math.inf, math.nan])
def test_rejects_speeds_that_are_not_finite_in_binary32(u_in):
    with pytest.raises(RangeError):
        GpuSolver.validate(LAYOUT, params(u_in=u_in))


def test_accepts_the_first_binary32_relaxation_time_above_one_half():
    GpuSolver.validate(LAYOUT, params(tau0=0.5 + 2.0 ** -24))


def test_rejects_population_indices_past_the_cell_limit():
    # 65536 x 65536 x 1 is 2^32 cells: past the reference's 32-bit indexing and
    # past this library's 2^32 - 64 cells
    with pytest.raises(RangeError):
        GpuSolver.validate((65536, 65536, 1), params())
    GpuSolver.validate((65536, 65535, 1), params())


def test_rejects_unknown_choices():
    for bad in (dict(operator="bgk"), dict(walls="ibb"), dict(precision="f64"), dict(lateral="open"),
                dict(kernel="warp"), dict(ramp_steps=-1)):
        with pytest.raises(RangeError):
            GpuSolver.validate(LAYOUT, params(**bad))
    # interpolated walls run with the one-cell-per-thread kernels and periodic faces only
    with pytest.raises(RangeError):
        GpuSolver.validate(LAYOUT, params(walls="bouzidi", kernel="tile"))
    with pytest.raises(RangeError):
        GpuSolver.validate(LAYOUT, params(walls="bouzidi", lateral="free-slip"))
