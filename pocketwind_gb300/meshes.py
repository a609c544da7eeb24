"""Host-side mesh generation and placement (the inputs of the voxelizer).

Mirrors the reference's mesh sources so the same triangles reach both the GPU
voxelizer and the CPU checker:

* ``loft``/``ahmed_mesh``/``stilts_mesh``/``cube_mesh``/``sphere_mesh`` follow
  src/geometry/presets.ts:38-184 (rectangular-station loft, Ahmed body with its
  100 mm nose radius and 25 degree slant, stilts, 100 mm cube, lat-long sphere);
* ``icosphere`` follows the test fixture generator
  tests/unit/voxelize/fixtures.ts:48-108 (icosahedron, midpoint subdivision);
* ``place_mesh``, ``default_orientation`` and ``default_length_cells`` follow
  src/geometry/transform.ts:31-143 (flow and up axes rotated onto +x and +z,
  scale by the longest extent, nose at nx/4, centred lateral axis, z centred or
  on the floor wall at z = 0.5; the dropped-mesh defaults).

Meshes are ``Mesh(positions: float32[9*T], triangle_count)`` in lattice cells.
Coordinates are computed in binary64 and stored in binary32, as the reference's
``Float32Array.set`` does.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from ._lib import RangeError


@dataclass
class Mesh:
    positions: np.ndarray  # float32, 9 per triangle
    triangle_count: int

    @staticmethod
    def from_triangles(tris) -> "Mesh":
        arr = np.asarray(tris, dtype=np.float64).reshape(-1, 9)
        return Mesh(arr.astype(np.float32).reshape(-1), arr.shape[0])

    def bounds(self):
        p = self.positions.reshape(-1, 3).astype(np.float64)
        return p.min(axis=0), p.max(axis=0)

    def translated(self, offset) -> "Mesh":
        p = self.positions.reshape(-1, 3).astype(np.float64) + np.asarray(offset, np.float64)
        return Mesh(p.astype(np.float32).reshape(-1), self.triangle_count)


def _hypot(*values: float) -> float:
    """Math.hypot as V8 evaluates it: scale by the largest magnitude and sum the
    squares with Kahan compensation."""
    mags = [abs(v) for v in values]
    top = max(mags)
    if top == 0:
        return 0.0
    total = 0.0
    comp = 0.0
    for m in mags:
        n = m / top
        summand = n * n - comp
        prelim = total + summand
        comp = (prelim - total) - summand
        total = prelim
    return math.sqrt(total) * top


# ----------------------------------------------------------------- presets.ts
def _quad(tris, a, b, c, d):
    tris.append((a, b, c))
    tris.append((a, c, d))


def loft(stations: Sequence[tuple]) -> Mesh:
    """Join rectangular stations (x, y_half, z_min, z_max) into a closed solid
    (presets.ts:61-79)."""
    rings = [[(x, -yh, z0), (x, yh, z0), (x, yh, z1), (x, -yh, z1)] for (x, yh, z0, z1) in stations]
    tris = []
    for k in range(len(rings) - 1):
        near, far = rings[k], rings[k + 1]
        for corner in range(4):
            nxt = (corner + 1) % 4
            _quad(tris, near[corner], far[corner], far[nxt], near[nxt])
    first, last = rings[0], rings[-1]
    _quad(tris, first[0], first[1], first[2], first[3])
    _quad(tris, last[0], last[3], last[2], last[1])
    return Mesh.from_triangles(tris)


def ahmed_mesh() -> Mesh:
    """Ahmed body above its stilts, in millimetres (presets.ts:86-109)."""
    radius, half_width, bottom = 100.0, 389.0 / 2, 50.0
    top = 50.0 + 288.0
    nose = []
    for seg in range(13):
        angle = (seg / 12) * (math.pi / 2)
        inset = radius * (1 - math.sin(angle))
        nose.append((radius * (1 - math.cos(angle)), half_width - inset, bottom + inset, top - inset))
    slant = (25 * math.pi) / 180
    slant_start = 1044 - 222 * math.cos(slant)
    slant_drop = 222 * math.sin(slant)
    return loft(nose + [(slant_start, half_width, bottom, top), (1044.0, half_width, bottom, top - slant_drop)])


def _cylinder(x, y, diameter, height, segments=16):
    r = diameter / 2
    tris = []

    def rim(z, s):
        th = (s / segments) * 2 * math.pi
        return (x + r * math.cos(th), y + r * math.sin(th), z)

    for s in range(segments):
        n = s + 1
        _quad(tris, rim(0, s), rim(0, n), rim(height, n), rim(height, s))
        tris.append(((x, y, 0), rim(0, n), rim(0, s)))
        tris.append(((x, y, height), rim(height, s), rim(height, n)))
    return tris


def stilts_mesh() -> Mesh:
    """The four 30 mm stilts under the Ahmed body (presets.ts:128-135)."""
    tris = []
    for x in (202.0, 672.0):
        for y in (-163.5, 163.5):
            tris += _cylinder(x, y, 30.0, 50.0)
    return Mesh.from_triangles(tris)


def cube_mesh() -> Mesh:
    return loft([(0.0, 50.0, 0.0, 100.0), (100.0, 50.0, 0.0, 100.0)])


def sphere_mesh() -> Mesh:
    """Latitude-longitude 100 mm sphere (presets.ts:146-170)."""
    radius, segs, rings = 50.0, 24, 16

    def vertex(ring, seg):
        phi = (ring / rings) * math.pi
        th = (seg / segs) * 2 * math.pi
        return (radius * math.sin(phi) * math.cos(th), radius * math.sin(phi) * math.sin(th), radius * math.cos(phi))

    tris = []
    for ring in range(rings):
        for seg in range(segs):
            nxt = (seg + 1) % segs
            top, bottom = vertex(ring, seg), vertex(ring + 1, seg)
            bottom_next, top_next = vertex(ring + 1, nxt), vertex(ring, nxt)
            if ring != 0:
                tris.append((top, bottom, top_next))
            if ring != rings - 1:
                tris.append((top_next, bottom, bottom_next))
    return Mesh.from_triangles(tris)


def preset_mesh(name: str) -> Optional[Mesh]:
    return {"ahmed-25": ahmed_mesh, "sphere": sphere_mesh, "cube": cube_mesh}.get(name, lambda: None)()


def preset_supports(name: str) -> Optional[Mesh]:
    return stilts_mesh() if name == "ahmed-25" else None


# ------------------------------------------------------------ icosphere fixture
def _unit(p):
    n = _hypot(*p)
    return (p[0] / n, p[1] / n, p[2] / n)


def icosphere(centre, radius: float, subdivisions: int = 5, extra_splits: int = 0) -> Mesh:
    """Seeded-shape icosphere of tests/unit/voxelize/fixtures.ts:48-108."""
    phi = (1 + math.sqrt(5)) / 2
    verts = [_unit(p) for p in [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi),
                                 (0, 1, phi), (0, -1, -phi), (0, 1, -phi), (phi, 0, -1), (phi, 0, 1),
                                 (-phi, 0, -1), (-phi, 0, 1)]]
    idx = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
           (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
           (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    faces = [(verts[a], verts[b], verts[c]) for a, b, c in idx]

    def mid(a, b):
        return _unit((a[0] + b[0], a[1] + b[1], a[2] + b[2]))

    def split(f):
        a, b, c = f
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        return [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]

    for _ in range(subdivisions):
        faces = [g for f in faces for g in split(f)]
    if extra_splits > 0:
        out = []
        for k, f in enumerate(faces):
            out.extend(split(f) if k < extra_splits else [f])
        faces = out
    arr = np.asarray(faces, np.float64).reshape(-1, 3)
    arr = arr * radius + np.asarray(centre, np.float64)
    return Mesh(arr.astype(np.float32).reshape(-1), len(faces))


# --------------------------------------------------------------- placement
# Placement and blockage limits of the tunnel (transform.ts:14-19).
NOSE_FRACTION_NX = 0.25
LENGTH_CAP_NX = 0.4
BLOCKAGE_MAX = 0.08
FLOOR_WALL_Z_CELLS = 0.5
_AXES = "xyz"


def _mesh_bounds(mesh: Mesh):
    """meshBounds (transform.ts:31-49): binary64 bounds of the float32 vertices."""
    if mesh.triangle_count < 1 or mesh.positions.size != 9 * mesh.triangle_count:
        raise RangeError("Mesh positions must match a positive triangle count.")
    p = mesh.positions.reshape(-1, 3).astype(np.float64)
    if not np.isfinite(p).all():
        raise RangeError("Mesh coordinates must be finite.")
    return p.min(axis=0), p.max(axis=0)


def _longest(extents) -> float:
    longest = float(max(extents))
    if longest == 0:
        raise RangeError("Mesh must have a nonzero extent.")
    return longest


def _check_layout(nx, ny, nz) -> None:
    for size in (nx, ny, nz):
        if isinstance(size, bool) or not float(size).is_integer() or size < 2 or size > 2 ** 53:
            raise RangeError("Grid dimensions must be integers of at least two cells.")


def default_orientation(mesh: Mesh):
    """defaultOrientation (transform.ts:70-74): z up, positive flow along the
    longer horizontal extent (x on ties).  Returns (flow_axis, flow_sign, up_axis)."""
    lo, hi = _mesh_bounds(mesh)
    ext = hi - lo
    return ("y" if ext[1] > ext[0] else "x"), 1, "z"


def default_length_cells(mesh: Mesh, nx: int, ny: int, nz: int, floor: bool) -> float:
    """defaultLengthCells (transform.ts:77-87): the body length in cells for a
    dropped mesh, capped at 0.4 nx and by an 8% blockage of its default
    orientation's frontal bounding box (rounded down to whole cells)."""
    del floor  # the reference takes it and does not use it
    _check_layout(nx, ny, nz)
    lo, hi = _mesh_bounds(mesh)
    ext = hi - lo
    longest = _longest(ext)
    frontal = min(ext[0], ext[1]) * ext[2]
    blockage = math.inf if frontal == 0 else math.floor(longest * math.sqrt(BLOCKAGE_MAX * ny * nz / frontal))
    return min(LENGTH_CAP_NX * nx, blockage)


def _lateral_axis(flow_axis: str, flow_sign: int, up_axis: str):
    """lateralAxis (transform.ts:89-100): the third axis, signed so that
    y = up x flow keeps every orientation right-handed."""
    if flow_axis not in _AXES or up_axis not in _AXES or flow_sign not in (1, -1):
        raise RangeError("Flow and up must be coordinate axes.")
    if flow_axis == up_axis:
        raise RangeError("Flow and up axes must differ.")
    axis = next(a for a in _AXES if a not in (flow_axis, up_axis))
    positive = (up_axis, flow_axis) in (("z", "x"), ("x", "y"), ("y", "z"))
    return _AXES.index(axis), (flow_sign if positive else -flow_sign)


def place_mesh(mesh: Mesh, nx: int, ny: int, nz: int, length_cells: float, floor: bool,
               supports: Optional[Mesh] = None, flow_axis: str = "x", flow_sign: int = 1, up_axis: str = "z"):
    """placeMesh (transform.ts:115-143): rotate flow_axis (sign flow_sign) onto
    lattice +x and up_axis onto +z, scale body and supports together so the
    body's longest extent spans length_cells, put the nose at nx / 4, centre
    the lateral axis, and centre z or rest the union of body and supports on
    the floor wall at z = 1/2.  Returns (body, supports or None)."""
    _check_layout(nx, ny, nz)
    if not (math.isfinite(length_cells) and length_cells > 0):
        raise RangeError("Body length in cells must be finite and positive.")
    lat, lat_sign = _lateral_axis(flow_axis, flow_sign, up_axis)
    fa, ua = _AXES.index(flow_axis), _AXES.index(up_axis)
    lo, hi = _mesh_bounds(mesh)
    sup_lo = _mesh_bounds(supports)[0] if supports is not None else None
    scale = length_cells / _longest(hi - lo)
    nose = lo[fa] if flow_sign == 1 else hi[fa]
    centre_y = (lo[lat] + hi[lat]) / 2
    centre_z = (lo[ua] + hi[ua]) / 2
    lowest = min(lo[ua], sup_lo[ua]) if sup_lo is not None else lo[ua]

    def tf(m: Mesh) -> Mesh:
        q = m.positions.reshape(-1, 3).astype(np.float64)
        out = np.empty_like(q)
        out[:, 0] = NOSE_FRACTION_NX * nx + flow_sign * (q[:, fa] - nose) * scale
        out[:, 1] = ny / 2 + lat_sign * (q[:, lat] - centre_y) * scale
        if floor:
            out[:, 2] = FLOOR_WALL_Z_CELLS + (q[:, ua] - lowest) * scale
        else:
            out[:, 2] = nz / 2 + (q[:, ua] - centre_z) * scale
        return Mesh(out.astype(np.float32).reshape(-1), m.triangle_count)

    return tf(mesh), (tf(supports) if supports is not None else None)


# ------------------------------------------------------- benchmark bodies
def bluff_body(length: float, width: float, height: float, nose_radius: float, slant_run: float,
               slant_deg: float = 25.0, segments: int = 12) -> Mesh:
    """Rounded-nose box with a rear slant, built like ahmedMesh (presets.ts:86-109)
    from cell dimensions: the nose stations inset the full section by the same
    radius, and the roof falls over the last ``slant_run`` cells at ``slant_deg``.
    Body frame: nose at x = 0, centred on y = 0, underside at z = 0."""
    half = width / 2
    nose = []
    for seg in range(segments + 1):
        angle = (seg / segments) * (math.pi / 2)
        inset = nose_radius * (1 - math.sin(angle))
        nose.append((nose_radius * (1 - math.cos(angle)), half - inset, inset, height - inset))
    drop = slant_run * math.tan(math.radians(slant_deg))
    return loft(nose + [(length - slant_run, half, 0.0, height), (length, half, 0.0, height - drop)])


def vehicle_case_mesh(nx: int, ny: int, scale: float = 1.0) -> Mesh:
    """The 40 x 15 x 11-cell body of the 128 x 64 x 64 vehicle case, with a
    25 degree slant over its last 8 cells and its underside 1.5 cells above the
    halfway floor wall (z = 0.5); ``scale`` enlarges every length (x4 for the
    512 x 256 x 256 case).  Nose at nx/4, centred in y."""
    body = bluff_body(40 * scale, 15 * scale, 11 * scale, 3 * scale, 8 * scale)
    return body.translated((0.25 * nx, ny / 2, 0.5 + 1.5 * scale))


def ellipsoid(centre, radii, subdivisions: int = 3) -> Mesh:
    m = icosphere((0, 0, 0), 1.0, subdivisions)
    p = m.positions.reshape(-1, 3).astype(np.float64) * np.asarray(radii, np.float64) + np.asarray(centre, np.float64)
    return Mesh(p.astype(np.float32).reshape(-1), m.triangle_count)


def yawed_box(centre, size, yaw_deg: float) -> Mesh:
    sx, sy, sz = (s / 2 for s in size)
    base = loft([(-sx, sy, -sz, sz), (sx, sy, -sz, sz)])
    p = base.positions.reshape(-1, 3).astype(np.float64)
    c, s = math.cos(math.radians(yaw_deg)), math.sin(math.radians(yaw_deg))
    rot = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    p = p @ rot.T + np.asarray(centre, np.float64)
    return Mesh(p.astype(np.float32).reshape(-1), base.triangle_count)
