"""VTK field export: host writer cases restating tests/unit/vtk.test.ts, the
lattice-to-physical scale and file name of src/io/field-export.ts, and on the
GPU the device-formatted body against the host writer, byte for byte."""
import struct

import numpy as np
import pytest

from pocketwind_gb300 import field_io as F
from pocketwind_gb300._lib import RangeError

NX = NY = NZ = 8
CELLS = NX * NY * NZ


def _field():
    cell = np.arange(CELLS, dtype=np.float64)
    rho = (cell + 0.5).astype(np.float32)
    vel = np.stack([cell, -cell, cell * 0.25], axis=1).astype(np.float32).reshape(-1)
    return rho, vel


def _bytes():
    rho, vel = _field()
    return F.write_vtk(NX, NY, NZ, 0.002, rho, vel)


def _rho_start(b):
    key = b"LOOKUP_TABLE default\n"
    return b.index(key) + len(key)


# vtk.test.ts:44-60
def test_header_lines():
    b = _bytes()
    assert b[:_rho_start(b)].decode().split("\n") == [
        "# vtk DataFile Version 3.0", "PocketWind field", "BINARY", "DATASET STRUCTURED_POINTS",
        "DIMENSIONS 8 8 8", "ORIGIN 0 0 0", "SPACING 0.002 0.002 0.002", "POINT_DATA 512",
        "SCALARS rho float 1", "LOOKUP_TABLE default", ""]


# vtk.test.ts:62-66
def test_densities_big_endian():
    b = _bytes()
    s = _rho_start(b)
    for cell in range(100):
        assert struct.unpack(">f", b[s + 4 * cell: s + 4 * cell + 4])[0] == cell + 0.5


# vtk.test.ts:68-80
def test_velocity_block_big_endian():
    b = _bytes()
    s = _rho_start(b)
    hdr = b"VECTORS velocity float\n"
    vs = s + CELLS * 4 + 1 + len(hdr)
    assert b[s + CELLS * 4] == 0x0A
    assert b[s + CELLS * 4 + 1: vs] == hdr
    for cell in range(100):
        x, y, z = struct.unpack(">3f", b[vs + 12 * cell: vs + 12 * cell + 12])
        assert (x, y, z) == (cell, -cell, cell * 0.25)


# vtk.test.ts:82-85
def test_single_trailing_newline():
    b = _bytes()
    vs = _rho_start(b) + CELLS * 4 + 1 + len(b"VECTORS velocity float\n")
    assert len(b) == vs + CELLS * 12 + 1 and b[-1] == 0x0A


# vtk.test.ts:87-93
def test_rejects_mismatched_arrays():
    rho, vel = _field()
    with pytest.raises(RangeError):
        F.write_vtk(NX, NY, NZ, 0.002, rho[:-1], vel)
    with pytest.raises(RangeError):
        F.write_vtk(NX, NY, NZ, 0.002, rho, vel[:-1])


# vtk.test.ts:95-100
def test_rejects_bad_grid():
    rho, vel = _field()
    with pytest.raises(RangeError):
        F.write_vtk(0, NY, NZ, 0.002, rho, vel)
    with pytest.raises(RangeError):
        F.write_vtk(NX, NY, 2.5, 0.002, rho, vel)
    with pytest.raises(RangeError):
        F.write_vtk(NX, NY, NZ, 0, rho, vel)
    for bad in (float("nan"), float("inf"), -0.002):
        with pytest.raises(RangeError):
            F.write_vtk(NX, NY, NZ, bad, rho, vel)


def test_number_formatting_follows_ecmascript():
    cases = {0.002: "0.002", 1.0: "1", 2: "2", 0.1 + 0.2: "0.30000000000000004", 1e-7: "1e-7",
             1.5e-7: "1.5e-7", 1e-6: "0.000001", 123e-20: "1.23e-18", 1e21: "1e+21", 1e20: "100000000000000000000",
             2.5e22: "2.5e+22", 0.5: "0.5", 12.25: "12.25", 1 / 3: "0.3333333333333333", -0.002: "-0.002"}
    for x, s in cases.items():
        assert F.js_number(x) == s, x


def test_lattice_to_field_scale():
    u = np.array([0.05, -0.025, 1e-3, 0.0123457], np.float32)
    got = F.lattice_to_field(u, 30.0)
    want = np.array([float(v) * (30.0 / 0.05) for v in u], np.float64).astype(np.float32)
    assert got.dtype == np.float32 and np.array_equal(got, want)
    assert got[0] == np.float32(30.0)
    for bad in (0, -1, float("nan"), float("inf")):
        with pytest.raises(RangeError):
            F.lattice_to_field(u, bad)


def test_field_vtk_bytes_is_writer_of_scaled_field():
    rho, vel = _field()
    a = F.field_vtk_bytes(NX, NY, NZ, 0.01, 20.0, rho, vel * np.float32(0.001))
    b = F.write_vtk(NX, NY, NZ, 0.01, rho, F.lattice_to_field(vel * np.float32(0.001), 20.0))
    assert a == b


def test_field_file_name():
    assert F.field_file_name("car") == "car-field.vtk"
    assert F.field_file_name('a/b\\c:d*e?f"g<h>i|j') == "a-b-c-d-e-f-g-h-i-j-field.vtk"
    assert F.field_file_name("   ") == "untitled-field.vtk"
    assert F.field_file_name("") == "untitled-field.vtk"
    assert F.field_file_name("  wing 2 \n") == "wing 2-field.vtk"
    assert F.field_file_name(" x　") == "x-field.vtk"


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_gpu_body_matches_host_writer(precision):
    from pocketwind_gb300 import geometry, solver
    from tests.shapes import blob_grid
    layout = (32, 32, 32)
    g, b = blob_grid("bb", layout)
    s = solver.GpuSolver.create(layout, geometry.grid_from_arrays(layout, g, b),
                                solver.SolverParams(tau0=0.8, u_in=0.06, precision=precision))
    s.step(37, True)
    m = s.macros()
    want = F.field_vtk_bytes(*layout, 0.004, 12.5, m[:, 0], m[:, 1:])
    got = F.solver_vtk(s, 0.004, 12.5)
    assert len(got) == len(want) and got == want
    with pytest.raises(RangeError):
        F.solver_vtk(s, 0.004, 0.0)
    s.destroy()


def test_field_export_known_file():
    """tests/unit/io/field-export.test.ts:23-61 on an 8^3 field: the inlet speed
    maps 0.05 to 20 m/s, the header, the first 100 densities and velocities read
    back big-endian, the file size, the unchanged source arrays, the refused
    speeds and the file names."""
    n, cells = 8, 512
    rho = (1 + np.arange(cells) / 1024).astype(np.float32)
    vel = np.tile(np.array([0.05, 0.025, -0.0125], np.float32), cells)
    source = vel.copy()
    field = F.lattice_to_field(vel, 20.0)
    assert list(field[:3]) == [20, 10, -5] and np.array_equal(vel, source)
    data = F.field_vtk_bytes(n, n, n, 0.004, 20.0, rho, vel)
    header = ("# vtk DataFile Version 3.0\nPocketWind field\nBINARY\nDATASET STRUCTURED_POINTS\n"
              "DIMENSIONS 8 8 8\nORIGIN 0 0 0\nSPACING 0.004 0.004 0.004\nPOINT_DATA 512\n"
              "SCALARS rho float 1\nLOOKUP_TABLE default\n").encode()
    assert data[:len(header)] == header
    v0 = len(header) + cells * 4 + 1 + len(b"VECTORS velocity float\n")
    for cell in range(100):
        assert struct.unpack_from(">f", data, len(header) + 4 * cell)[0] == np.float32(1 + cell / 1024)
        assert struct.unpack_from(">3f", data, v0 + 12 * cell) == (20.0, 10.0, -5.0)
    assert len(data) == v0 + cells * 12 + 1
    for bad in (0.0, float("nan")):
        with pytest.raises(RangeError):
            F.lattice_to_field(vel, bad)
    assert F.field_file_name("Ahmed 25") == "Ahmed 25-field.vtk"
    assert F.field_file_name("a/b:c") == "a-b-c-field.vtk"
    assert F.field_file_name("  ") == "untitled-field.vtk"
