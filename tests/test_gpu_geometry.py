"""GPU voxelizer parity: the packed geometry and boundary list equal the binary64
restatement of src/geometry/voxelize.ts + wall-links.ts bit for bit, with the
halfway fractions of linkFractions: false and with measured link fractions
(triangle-bins.ts), on the reference's own test meshes and on the benchmark
bodies."""
import numpy as np
import pytest

from oracle import oracle as O
from pocketwind_gb300 import meshes
from tests.shapes import box

pytestmark = pytest.mark.gpu


def _both(body, supports, layout, floor, link_fractions=False):
    from pocketwind_gb300.geometry import voxelize
    g = voxelize(body, supports, layout, floor, link_fractions=link_fractions)
    r = O.voxelize(body.positions, None if supports is None else supports.positions, layout, floor,
                   link_fractions=link_fractions)
    return g, r


CASES = [
    ("icosphere r20", lambda: (meshes.icosphere((32, 32, 32), 20), None), (64, 64, 64), False),
    ("cube 8000", lambda: (box([20.2] * 3, [40.2] * 3), None), (64, 64, 64), False),
    ("open cube", lambda: (box([20.2] * 3, [40.2] * 3, True), None), (64, 64, 64), False),
    ("thin plate", lambda: (box([20.2] * 3, [20.5, 40.2, 40.2]), None), (64, 64, 64), False),
    ("body and support", lambda: (box([20.2] * 3, [24.2] * 3), box([22.2, 22.2, 18.2], [26.2, 26.2, 22.2])),
     (64, 64, 64), False),
    ("floor corners", lambda: (box([20.25] * 3, [24.25] * 3), box([30.25] * 3, [34.25] * 3)), (64, 64, 64), True),
    ("sphere case 96x48x48", lambda: (meshes.icosphere((24, 24, 24), 6, 4), None), (96, 48, 48), False),
    ("vehicle case 128x64x64", lambda: (meshes.vehicle_case_mesh(128, 64), None), (128, 64, 64), True),
    ("ahmed preset with stilts", lambda: meshes.place_mesh(meshes.ahmed_mesh(), 128, 64, 64, 48, True,
                                                           meshes.stilts_mesh()), (128, 64, 64), True),
    ("empty tunnel", lambda: (meshes.Mesh(np.zeros(0, np.float32), 0), None), (16, 8, 8), True),
]


@pytest.mark.parametrize("measure", [False, True], ids=["halfway", "measured"])
@pytest.mark.parametrize("name,make,layout,floor", CASES, ids=[c[0] for c in CASES])
def test_voxelizer_bit_exact(name, make, layout, floor, measure):
    body, supports = make()
    g, r = _both(body, supports, layout, floor, measure)
    assert np.array_equal(g.geometry, r.geometry)
    assert g.missed_links == r.missed_links
    assert np.array_equal(g.boundary_cells, r.boundary_cells)
    assert (g.solid_cells, g.frontal_cells, g.watertight) == (r.solid_cells, r.frontal_cells, r.watertight)
    assert g.blockage == r.blockage


def test_voxelizer_rejects_invalid_inputs():
    from pocketwind_gb300._lib import RangeError
    from pocketwind_gb300.geometry import voxelize
    mesh = box([20] * 3, [24] * 3)
    with pytest.raises(RangeError):
        voxelize(mesh, None, (1, 64, 64), False)
    bad = mesh.positions.copy()
    bad[0] = np.nan
    with pytest.raises(RangeError):
        voxelize(mesh, meshes.Mesh(bad, mesh.triangle_count), (64, 64, 64), False)


def test_winding_invariance_on_gpu():
    from pocketwind_gb300.geometry import voxelize
    mesh = box([20] * 3, [24] * 3)
    rev = mesh.positions.reshape(-1, 3, 3)[:, [0, 2, 1], :].reshape(-1).copy()
    a = voxelize(mesh, None, (64, 64, 64), False)
    b = voxelize(meshes.Mesh(rev, mesh.triangle_count), None, (64, 64, 64), False)
    assert a.solid_cells == 64 and np.array_equal(a.geometry, b.geometry)
