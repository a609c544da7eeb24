"""Solver-state checkpoint and restore: a run that is saved, restored into a
fresh domain and stepped on gives the same populations, macros and drag as the
run that went on without stopping, bit for bit; damaged or mismatched blobs
are refused and leave the domain untouched."""
import numpy as np
import pytest

from tests.shapes import blob_grid

pytestmark = pytest.mark.gpu
LAYOUT = (32, 32, 32)


def _solver(precision="f16", op="reg", les=True, kernel="auto", lateral="periodic", tau0=0.8, ramp=0, walls="bb",
            strict=False):
    from pocketwind_gb300 import geometry, solver
    g, b = blob_grid(walls, LAYOUT)
    return solver.GpuSolver.create(LAYOUT, geometry.grid_from_arrays(LAYOUT, g, b),
                                   solver.SolverParams(tau0=tau0, u_in=0.06, les=les, operator=op, precision=precision,
                                                       kernel=kernel, lateral=lateral, ramp_steps=ramp, walls=walls,
                                                       strict=strict))


@pytest.mark.parametrize("precision,kernel,lateral,first,walls,strict", [
    ("f16", "auto", "periodic", 41, "bb", False), ("f32", "auto", "free-slip", 40, "bb", False),
    ("bf16", "tile", "periodic", 13, "bb", False), ("f32", "auto", "periodic", 7, "bb", False),
    ("f16", "auto", "periodic", 21, "bouzidi", False), ("f32", "auto", "periodic", 30, "bouzidi", True)])
def test_restore_continues_bit_exact(precision, kernel, lateral, first, walls, strict):
    ramp = 20 if first == 7 else 0
    a = _solver(precision, kernel=kernel, lateral=lateral, ramp=ramp, walls=walls, strict=strict)
    a.step(first, True)
    blob = a.save_checkpoint()
    a.step(33, True)
    a.encode_force()
    fa = a.read_force()
    b = _solver(precision, kernel=kernel, lateral=lateral, ramp=ramp, walls=walls, strict=strict)
    b.step(5)
    b.load_checkpoint(blob)
    assert b.step_count == first
    b.step(33, True)
    b.encode_force()
    fb = b.read_force()
    assert np.array_equal(a.populations_raw(), b.populations_raw())
    assert np.array_equal(a.macros(), b.macros())
    assert (fa.step, fa.fx, fa.fy, fa.fz) == (fb.step, fb.fx, fb.fy, fb.fz)
    a.destroy()
    b.destroy()


def test_restored_force_and_macros_before_stepping():
    a = _solver()
    a.step(20, True)
    blob = a.save_checkpoint()
    a.encode_force()
    fa = a.read_force()
    b = _solver()
    b.load_checkpoint(blob)
    b.encode_force()
    fb = b.read_force()
    assert (fa.fx, fa.fy, fa.fz) == (fb.fx, fb.fy, fb.fz)
    assert np.array_equal(a.macros(), b.macros())
    a.destroy()
    b.destroy()


def test_bad_blobs_are_refused_and_leave_the_state():
    from pocketwind_gb300._lib import RangeError
    a = _solver()
    a.step(10, True)
    blob = bytearray(a.save_checkpoint())
    b = _solver()
    b.step(3, True)
    before = b.populations_raw()
    bad = [bytes(blob[:-1]), bytes(blob[:50]), b"nonsense" * 20]
    flipped = bytearray(blob)
    flipped[200] ^= 1
    bad.append(bytes(flipped))
    wrong_steps = bytearray(blob)
    wrong_steps[60] ^= 1  # the step count: the checksum covers the header too
    bad.append(bytes(wrong_steps))
    for blob_bad in bad:
        with pytest.raises(RangeError):
            b.load_checkpoint(blob_bad)
        assert b.step_count == 3
        assert np.array_equal(b.populations_raw(), before)
    other = _solver(precision="f32")
    with pytest.raises(RangeError):
        other.load_checkpoint(bytes(blob))
    other_tau = _solver(tau0=0.7)
    with pytest.raises(RangeError):
        other_tau.load_checkpoint(bytes(blob))
    for s in (a, b, other, other_tau):
        s.destroy()
