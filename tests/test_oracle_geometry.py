"""Pin the voxelizer and wall-link restatement to the reference's golden values.

Restates tests/unit/voxelize/voxelize.test.ts and
tests/unit/wall-links/wall-links.test.ts against the binary64 oracle.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from pocketwind_gb300.meshes import Mesh, icosphere
from tests.shapes import C, EQ, FLOOR, FLUID, NO_Q, SOLID, SUPPORT, box

LAYOUT = (64, 64, 64)
CELLS = 64 ** 3
idx = lambda x, y, z: x + 64 * (y + 64 * z)


def vox(body, supports=None, floor=False, link_fractions=True, layout=LAYOUT):
    return O.voxelize(None if body is None else body.positions,
                      None if supports is None else supports.positions, layout, floor, link_fractions)


def test_empty_tunnel_keeps_boundaries():
    """voxelize.test.ts:10-27"""
    for floor in (False, True):
        g = vox(Mesh(np.zeros(0, np.float32), 0), floor=floor, link_fractions=False)
        assert g.solid_cells == 0 and g.frontal_cells == 0 and g.boundary_cells.size == 0
        kinds = g.geometry[:CELLS] & 7
        assert (kinds == EQ).any()
        assert (kinds == FLOOR).any() == floor


def test_sphere_volume_and_frontal_area():
    """voxelize.test.ts:29-35"""
    g = vox(icosphere((32, 32, 32), 20))
    assert g.watertight
    assert abs(g.solid_cells / (4 / 3 * math.pi * 20 ** 3) - 1) < 0.02
    assert abs(g.frontal_cells / (math.pi * 20 ** 2) - 1) < 0.03
    assert g.blockage == g.frontal_cells / (64 * 64)


def test_cube_exact_and_majority_vote_with_missing_face():
    """voxelize.test.ts:37-49"""
    closed = vox(box([20.2] * 3, [40.2] * 3))
    open_ = vox(box([20.2] * 3, [40.2] * 3, True))
    assert closed.watertight and closed.solid_cells == 8000
    assert not open_.watertight
    assert abs(open_.solid_cells / closed.solid_cells - 1) < 0.05
    assert open_.missed_links > 0


def test_thin_plate_is_not_inflated():
    """voxelize.test.ts:51-59"""
    g = vox(box([20.2, 20.2, 20.2], [20.5, 40.2, 40.2]))
    assert g.solid_cells == 0 and g.frontal_cells == 0 and g.boundary_cells.size == 0 and g.watertight


def test_body_precedence_and_support_blockage():
    """voxelize.test.ts:61-73"""
    g = vox(box([20.2] * 3, [24.2] * 3), box([22.2, 22.2, 18.2], [26.2, 26.2, 22.2]))
    assert g.solid_cells == 64 and g.frontal_cells == 16 and g.blockage == 28 / (64 * 64)
    assert g.geometry[idx(23, 23, 21)] & 7 == SOLID
    assert g.geometry[idx(25, 25, 19)] & 7 == SUPPORT


def test_eq_faces_and_floor_corners():
    """voxelize.test.ts:75-86"""
    mesh = box([20.2] * 3, [24.2] * 3)
    g = vox(mesh, floor=True)
    assert g.geometry[idx(0, 4, 0)] == FLOOR and g.geometry[idx(63, 4, 0)] == FLOOR
    assert g.geometry[idx(0, 4, 4)] == EQ and g.geometry[idx(63, 4, 4)] == EQ
    assert g.geometry[idx(4, 4, 63)] == EQ
    p = vox(mesh)
    assert p.geometry[idx(4, 4, 0)] == FLUID and p.geometry[idx(4, 4, 63)] == FLUID


def test_winding_invariance():
    """voxelize.test.ts:90-103"""
    mesh = box([20] * 3, [24] * 3)
    t = mesh.positions.reshape(-1, 3, 3).copy()
    rev = t[:, [0, 2, 1], :].reshape(-1)
    fwd = vox(mesh)
    bwd = vox(Mesh(rev.astype(np.float32), mesh.triangle_count))
    assert fwd.solid_cells == 64 and fwd.watertight
    assert np.array_equal(fwd.geometry, bwd.geometry) and bwd.watertight


def test_open_support_not_watertight_and_invalid_inputs():
    """voxelize.test.ts:105-126"""
    g = vox(box([20] * 3, [24] * 3), box([30.2] * 3, [34.2] * 3, True))
    assert not g.watertight
    mesh = box([20] * 3, [24] * 3)
    with pytest.raises(ValueError):
        vox(mesh, layout=(1, 64, 64))
    bad = mesh.positions.copy()
    bad[0] = np.nan
    with pytest.raises(ValueError):
        O.voxelize(mesh.positions, bad, LAYOUT, False)


def _analytic_q(origin, d, centre, radius):
    d = [-v for v in d]
    rel = [o - c for o, c in zip(origin, centre)]
    a = sum(v * v for v in d)
    b = 2 * sum(r * v for r, v in zip(rel, d))
    c = sum(r * r for r in rel) - radius * radius
    return (-b - math.sqrt(b * b - 4 * a * c)) / (2 * a)


@pytest.mark.slow
def test_sphere_links_match_analytic_ray_sphere():
    """wall-links.test.ts:40-95"""
    centre, radius = (31.37, 30.23, 32.41), 20
    mesh = icosphere(centre, radius, 5)
    assert mesh.triangle_count == 20480
    g = vox(mesh)
    q = g.geometry[2 * CELLS:].view(np.float32)
    checked = analytic = 0
    max_radial = max_q = 0.0
    for cell in g.boundary_cells:
        flag = int(g.geometry[cell])
        base = int(g.geometry[CELLS + cell])
        assert base != NO_Q
        origin = (cell % 64, (cell // 64) % 64, cell // 4096)
        off = 0
        for i in range(19):
            if not flag & (1 << (3 + i)):
                continue
            d = C[i]
            exp = _analytic_q(origin, d, centre, radius)
            act = float(q[base + off])
            rd = math.dist([origin[a] - act * d[a] for a in range(3)], centre)
            max_radial = max(max_radial, abs(rd - radius))
            hit = [origin[a] - exp * d[a] - centre[a] for a in range(3)]
            cosine = abs(sum(hit[a] * d[a] for a in range(3))) / (radius * math.hypot(*d))
            if 0 <= exp <= 1 and cosine >= 0.6:
                max_q = max(max_q, abs(act - exp))
                analytic += 1
            assert 0.001 - 1e-9 <= act <= 1
            off += 1
            checked += 1
    assert checked > 10000 and analytic > 0
    assert max_radial < 0.02 and max_q < 0.02 and g.missed_links == 0 and q.size == checked


def test_packing_of_masks_offsets_and_boundary():
    """wall-links.test.ts:97-138"""
    g = vox(box([20.25] * 3, [24.25] * 3), box([30.25] * 3, [34.25] * 3), floor=True)
    q = g.geometry[2 * CELLS:].view(np.float32)
    kinds = g.geometry[:CELLS] & 7
    boundary = set(int(c) for c in g.boundary_cells)
    next_base = floor_links = support_links = 0
    for cell in range(CELLS):
        x, y, z = cell % 64, (cell // 64) % 64, cell // 4096
        links = []
        if kinds[cell] == FLUID:
            for i in range(1, 19):
                sx, sy, sz = x - C[i][0], (y - C[i][1] + 64) % 64, z - C[i][2]
                t = EQ if (sx < 0 or sx >= 64 or sz < 0 or sz >= 64) else int(kinds[sx + 64 * (sy + 64 * sz)])
                if SOLID <= t <= FLOOR:
                    links.append((i, t))
        mask = sum(1 << (3 + i) for i, _ in links)
        assert (int(g.geometry[cell]) & ~7) == mask
        assert (cell in boundary) == any(t == SOLID for _, t in links)
        assert int(g.geometry[CELLS + cell]) == (NO_Q if not links else next_base)
        for k, (_, t) in enumerate(links):
            if t == FLOOR:
                assert q[next_base + k] == 0.5
                floor_links += 1
            if t == SUPPORT:
                support_links += 1
        next_base += len(links)
    assert q.size == next_base and floor_links > 0 and support_links > 0 and g.missed_links == 0


def test_halfway_fractions_when_not_measuring():
    """wall-links.test.ts:140-153"""
    mesh = box([20.25] * 3, [24.25] * 3)
    measured = vox(mesh)
    halfway = vox(mesh, link_fractions=False)
    assert np.array_equal(halfway.geometry[:2 * CELLS], measured.geometry[:2 * CELLS])
    assert halfway.geometry.size == measured.geometry.size
    assert np.array_equal(halfway.boundary_cells, measured.boundary_cells)
    q = halfway.geometry[2 * CELLS:].view(np.float32)
    assert q.size > 0 and np.all(q == 0.5) and halfway.missed_links == 0


def test_nearest_link_hits():
    """wall-links.test.ts:155-162"""
    mesh = box([4, 4, 4], [4.75, 8, 8]).positions
    L = (16, 16, 16)
    assert abs(O.nearest_link_hit(mesh, L, (3.5, 6, 6), (1, 0, 0)) - 0.5) < 5e-3
    assert abs(O.nearest_link_hit(mesh, L, (5, 6, 6), (-1, 0, 0)) - 0.25) < 5e-3
    assert abs(O.nearest_link_hit(mesh, L, (3, 6, 6), (1, 0, 0)) - 1) < 5e-3
    assert O.nearest_link_hit(mesh, L, (3, 6, 6), (-1, 0, 0)) is None


@pytest.mark.parametrize("axis", [1, 2])
def test_periodic_image_links(axis):
    """wall-links.test.ts:166-189"""
    lo, hi = [20.2] * 3, [24.2] * 3
    lo[axis], hi[axis] = 60.2, 63.2
    g = vox(box(lo, hi))
    p = [22, 22, 22]
    p[axis] = 0
    cell = p[0] + 64 * (p[1] + 64 * p[2])
    q = g.geometry[2 * CELLS:].view(np.float32)
    off = int(g.geometry[CELLS + cell])
    checked = 0
    for i in range(19):
        if not int(g.geometry[cell]) & (1 << (3 + i)):
            continue
        if C[i][axis] == 1:
            assert abs(q[off] - 0.8) < 5e-5
            checked += 1
        off += 1
    assert checked == 5 and g.missed_links == 0


def test_wall_clamped_close_to_fluid_centre():
    """wall-links.test.ts:191-199"""
    g = vox(box([20.0001, 20.2, 20.2], [24.2] * 3))
    cell = 20 + 64 * (22 + 64 * 22)
    base = int(g.geometry[CELLS + cell])
    assert abs(g.geometry[2 * CELLS:].view(np.float32)[base] - 0.001) < 5e-7


def test_missing_intersections_counted():
    """wall-links.test.ts:202-210"""
    flags = np.zeros(CELLS, np.uint32)
    flags[32 + 64 * (32 + 64 * 32)] = SOLID
    geometry, boundary, missed = O.build_wall_links(flags, box([10] * 3, [12] * 3).positions, None,
                                                    LAYOUT, False)
    assert boundary.size == 18 and missed == 18
    assert np.all(geometry[2 * CELLS:].view(np.float32) == 0.5) and geometry.size == 2 * CELLS + 18
