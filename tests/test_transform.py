"""Mesh placement on the CPU, restating tests/unit/transform.test.ts
(placeMesh, defaultOrientation, defaultLengthCells; src/geometry/transform.ts)
with the reference's binary cube fixture."""
import math

import numpy as np
import pytest

from pocketwind_gb300 import meshes
from pocketwind_gb300._lib import RangeError
from tests.shapes import _cube

LAYOUT = (256, 128, 128)


def cube() -> meshes.Mesh:
    """The reference's tests/fixtures/stl/cube-binary.stl: the unit cube, 12 triangles."""
    positions = _cube()
    return meshes.Mesh(positions.reshape(-1), positions.size // 9)


def box(x, y, z, offset=(0, 0, 0)) -> meshes.Mesh:
    c = cube()
    p = c.positions.reshape(-1, 3).astype(np.float64) * np.array([x, y, z]) + np.array(offset, np.float64)
    return meshes.Mesh(p.astype(np.float32).reshape(-1), c.triangle_count)


def bounds(mesh):
    p = mesh.positions.reshape(-1, 3)
    return [[float(p[:, a].min()), float(p[:, a].max())] for a in range(3)]


def place(mesh, length, floor=False, **kw):
    return meshes.place_mesh(mesh, *LAYOUT, length, floor, **kw)


def test_places_the_cube_nose_at_a_quarter_of_nx_and_centres_y_and_z():
    source = cube()
    original = source.positions.copy()
    body, supports = place(source, 40)
    assert bounds(body) == [[64, 104], [44, 84], [44, 84]]
    assert body.triangle_count == 12 and supports is None
    assert np.array_equal(source.positions, original)


def test_reversed_flow_keeps_the_nose_and_the_scale():
    mesh = box(10, 4, 2, (20, -3, 7))
    forward, _ = place(mesh, 40)
    reverse, _ = place(mesh, 40, flow_sign=-1)
    assert bounds(forward) == bounds(reverse)
    assert np.all(forward.positions[0::3] + reverse.positions[0::3] == 168)


def test_scales_by_the_longest_dimension_even_when_vertical():
    body, _ = place(box(2, 4, 10), 40)
    assert bounds(body) == [[64, 72], [56, 72], [44, 84]]


def test_rotates_y_flow_to_lattice_x_with_z_up():
    mesh = box(10, 30, 5)
    flow_axis, flow_sign, up_axis = meshes.default_orientation(mesh)
    body, _ = place(mesh, 60, flow_axis=flow_axis, flow_sign=flow_sign, up_axis=up_axis)
    assert bounds(body) == [[64, 124], [54, 74], [59, 69]]


@pytest.mark.parametrize("flow_axis", "xyz")
@pytest.mark.parametrize("up_axis", "xyz")
@pytest.mark.parametrize("flow_sign", [-1, 1])
def test_every_orientation_is_a_proper_rotation(flow_axis, up_axis, flow_sign):
    if flow_axis == up_axis:
        return
    mesh = meshes.Mesh(np.array([0, 0, 0, 1, 0, 0, 0, 1, 1], np.float32), 1)
    body, _ = meshes.place_mesh(mesh, *LAYOUT, 1, False, flow_axis=flow_axis, flow_sign=flow_sign,
                                up_axis=up_axis)
    up = "xyz".index(up_axis)
    for v in range(3):
        assert body.positions[3 * v + 2] == np.float32(63.5 + float(mesh.positions[3 * v + up]))
    # the cross product's component along up survives a proper rotation
    p = body.positions.astype(np.float64)
    ax, ay = p[3] - p[0], p[4] - p[1]
    bx, by = p[6] - p[0], p[7] - p[1]
    assert ax * by - ay * bx + 0.0 == {"x": 0.0, "y": -1.0, "z": 1.0}[up_axis]


def test_places_body_and_supports_with_one_transform_on_the_floor():
    mesh = box(10, 4, 2, (0, 0, 5))
    supports = box(2, 2, 5, (2, 1, 0))
    original = supports.positions.copy()
    body, placed = place(mesh, 40, True, supports=supports)
    assert bounds(body) == [[64, 104], [56, 72], [20.5, 28.5]]
    assert bounds(placed) == [[72, 80], [60, 68], [0.5, 20.5]]
    assert np.array_equal(supports.positions, original)


def test_rests_the_body_on_the_floor_without_supports():
    body, _ = place(box(10, 4, 2, (10, -8, 20)), 40, True)
    assert bounds(body) == [[64, 104], [56, 72], [0.5, 8.5]]


def test_rejects_parallel_axes_and_invalid_lengths():
    with pytest.raises(RangeError):
        place(cube(), 40, up_axis="x")
    for length in (0, -1, math.nan, math.inf):
        with pytest.raises(RangeError):
            place(cube(), length)


def test_default_orientation_takes_the_longest_horizontal_extent():
    assert meshes.default_orientation(box(10, 30, 5)) == ("y", 1, "z")
    assert meshes.default_orientation(box(30, 10, 5)) == ("x", 1, "z")
    assert meshes.default_orientation(box(10, 10, 30)) == ("x", 1, "z")


def test_default_length_caps_a_sphere_box_at_36_cells():
    sphere = meshes.Mesh(np.array([-150, 0, 0, 150, 0, 0, 0, -150, 0,
                                   0, 150, 0, 0, 0, -150, 0, 0, 150], np.float32), 2)
    for floor in (True, False):
        length = meshes.default_length_cells(sphere, *LAYOUT, floor)
        assert length == 36
        assert length ** 2 / (LAYOUT[1] * LAYOUT[2]) <= 0.08


def test_default_length_uses_the_blockage_or_the_length_cap():
    ahmed = box(1044, 389, 288)
    block = math.floor(math.sqrt(0.08 * 128 * 128 / (389 * 288)) * 1044)
    assert meshes.default_length_cells(ahmed, *LAYOUT, True) == min(0.4 * 256, block)
    assert meshes.default_length_cells(box(1000, 1, 1), *LAYOUT, False) == 0.4 * 256
    # y-oriented and tall bodies are sized by their longest dimension
    assert (meshes.default_length_cells(box(389, 1044, 288), *LAYOUT, False)
            == meshes.default_length_cells(box(1044, 389, 288), *LAYOUT, False))
    assert meshes.default_length_cells(box(1, 1, 10), *LAYOUT, False) == 102.4
