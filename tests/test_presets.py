"""Preset bodies on the CPU, restating tests/unit/presets.test.ts: the Ahmed body's
size, stilts, rounded nose and 25 degree slant, the cube and the sphere, and
that each placed preset voxelizes as a closed surface (through the binary64
voxelizer restatement, which the GPU voxelizer equals bit for bit)."""
import math

import numpy as np

from oracle import oracle as O
from pocketwind_gb300 import meshes


def extent(mesh):
    p = mesh.positions.reshape(-1, 3).astype(np.float64)
    return p.min(axis=0), p.max(axis=0) - p.min(axis=0)


def test_ahmed_body_at_its_reference_size():
    lo, size = extent(meshes.preset_mesh("ahmed-25"))
    assert list(size) == [1044, 389, 288]
    assert lo[2] == 50  # lifted 50 mm onto the stilts


def test_ahmed_stilts():
    lo, size = extent(meshes.preset_supports("ahmed-25"))
    assert lo[2] == 0 and size[2] == 50
    assert math.isclose(size[0], 672 - 202 + 30, abs_tol=1e-9)
    assert math.isclose(size[1], 2 * 163.5 + 30, abs_tol=1e-9)
    assert meshes.preset_supports("sphere") is None


def test_ahmed_nose_edges_take_the_100_mm_radius():
    p = meshes.preset_mesh("ahmed-25").positions.reshape(-1, 3)
    nose = p[p[:, 0] == 0]
    assert [nose[:, 1].min(), nose[:, 1].max()] == [-94.5, 94.5]
    assert [nose[:, 2].min(), nose[:, 2].max()] == [150, 238]


def test_ahmed_rear_slant_is_222_mm_at_25_degrees():
    p = meshes.preset_mesh("ahmed-25").positions.reshape(-1, 3)
    base_top = float(p[p[:, 0] == 1044][:, 2].max())
    assert math.isclose(base_top, 338 - 222 * math.sin(25 * math.pi / 180), abs_tol=1e-4)


def test_cube_and_sphere_and_unknown_presets():
    assert list(extent(meshes.preset_mesh("cube"))[1]) == [100, 100, 100]
    assert [round(v) for v in extent(meshes.preset_mesh("sphere"))[1]] == [100, 100, 100]
    assert meshes.preset_mesh("custom") is None and meshes.preset_mesh("missing") is None


def _voxelize(name, layout, length, floor):
    body, supports = meshes.place_mesh(meshes.preset_mesh(name), *layout, length, floor,
                                       supports=meshes.preset_supports(name))
    return O.voxelize(body.positions, None if supports is None else supports.positions, layout, floor,
                      link_fractions=False)


def test_presets_voxelize_as_closed_surfaces():
    ahmed = _voxelize("ahmed-25", (64, 32, 32), 32, True)
    assert ahmed.watertight and ahmed.solid_cells > 0
    cube = _voxelize("cube", (32, 32, 32), 8, False)
    assert cube.watertight and cube.solid_cells == 8 * 8 * 8
    sphere = _voxelize("sphere", (32, 32, 32), 12, False)
    assert sphere.watertight and sphere.solid_cells > 0


def _canonical_stl(mesh) -> bytes:
    """The reference's canonical binary STL (scripts/stl-canonical.ts and
    export-geometry.ts): an 80-byte header starting "pocketwind preset geometry",
    the count, then per triangle a zero normal, the nine float32 coordinates
    (negative zero written as zero) and a zero attribute."""
    import struct
    out = bytearray(84 + 50 * mesh.triangle_count)
    header = b"pocketwind preset geometry"
    out[:len(header)] = header
    struct.pack_into("<I", out, 80, mesh.triangle_count)
    p = mesh.positions.astype(np.float32).copy()
    p[p == 0] = 0.0
    for t in range(mesh.triangle_count):
        start = 84 + 50 * t + 12
        out[start:start + 36] = p[9 * t:9 * t + 9].astype("<f4").tobytes()
    return bytes(out)


def test_presets_equal_the_reference_geometry_byte_for_byte():
    """The preset generators reproduce the reference's published bodies
    (public/validation/geometry/*.stl, checksums in tests/golden/preset_geometry.json)."""
    import hashlib
    import json
    from pathlib import Path
    sums = json.loads((Path(__file__).parent / "golden" / "preset_geometry.json").read_text())["sha256"]
    for name, mesh in (("ahmed-25.stl", meshes.preset_mesh("ahmed-25")), ("cube.stl", meshes.preset_mesh("cube")),
                       ("sphere.stl", meshes.preset_mesh("sphere")),
                       ("stilts.stl", meshes.preset_supports("ahmed-25"))):
        assert hashlib.sha256(_canonical_stl(mesh)).hexdigest() == sums[name], name
