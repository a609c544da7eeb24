"""Voxel grids: the reference's ``voxelize`` and ``VoxelGrid`` on the GPU.

``voxelize(body, supports, layout, floor)`` mirrors src/geometry/voxelize.ts:172-199
with ``linkFractions: false`` (the halfway-wall path the solver uses,
src/app/run.ts:188-191): it runs the library's parity-ray voxelizer and returns a
``VoxelGrid`` whose packed ``geometry`` (flags, q offsets, f32 fractions) and
``boundary_cells`` match src/geometry/voxel-grid.ts:7-15.  The device copy stays
resident for ``GpuSolver.create``; the host arrays are read back on first use.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib
from .meshes import Mesh

FLUID, SOLID, SUPPORT, FLOOR, EQ = range(5)
CELL_TYPE_MASK = 7
NO_Q = 0xFFFFFFFF


class _GridHandle:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if self.ptr:
            _lib.load().pw_grid_destroy(self.ptr)
            self.ptr = None


@dataclass
class VoxelGrid:
    nx: int
    ny: int
    nz: int
    solid_cells: int
    frontal_cells: int
    blockage: float
    watertight: bool
    missed_links: int
    geometry_len: int
    boundary_count: int
    _handle: _GridHandle = field(repr=False)
    _geometry: Optional[np.ndarray] = field(default=None, repr=False)
    _boundary: Optional[np.ndarray] = field(default=None, repr=False)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def geometry(self) -> np.ndarray:
        if self._geometry is None:
            out = np.empty(self.geometry_len, np.uint32)
            _lib.check(_lib.load().pw_grid_read_geometry(self._handle.ptr, out.ctypes.data_as(C.c_void_p), out.size),
                       "read geometry")
            self._geometry = out
        return self._geometry

    @property
    def boundary_cells(self) -> np.ndarray:
        if self._boundary is None:
            out = np.empty(max(self.boundary_count, 1), np.uint32)
            _lib.check(_lib.load().pw_grid_read_boundary(self._handle.ptr, out.ctypes.data_as(C.c_void_p),
                                                         out.size), "read boundary")
            self._boundary = out[: self.boundary_count]
        return self._boundary

    @property
    def flags(self) -> np.ndarray:
        return self.geometry[: self.cells]


def _from_handle(ptr) -> VoxelGrid:
    st = _lib.GridStats()
    _lib.check(_lib.load().pw_grid_stats_get(ptr, C.byref(st)), "grid stats")
    return VoxelGrid(st.nx, st.ny, st.nz, st.solid_cells, st.frontal_cells, st.blockage, bool(st.watertight),
                     st.missed_links, int(st.geometry_len), int(st.boundary_cells), _GridHandle(ptr))


def _mesh_array(m) -> tuple:
    if m is None:
        return None, 0
    if isinstance(m, Mesh):
        a = np.ascontiguousarray(m.positions, np.float32)
    else:
        a = np.ascontiguousarray(m, np.float32).reshape(-1)
    if a.size % 9:
        raise _lib.RangeError("Mesh positions must match a non-negative triangle count.")
    return a, a.size // 9


def voxelize(body, supports, layout, floor: bool, link_fractions: bool = False) -> VoxelGrid:
    """GPU voxelize (voxelize.ts:172); link_fractions measures each wall link's
    fraction for interpolated walls (wall-links.ts:53-80), otherwise every
    fraction is the halfway value 1/2."""
    nx, ny, nz = (int(v) for v in layout)
    for v, orig in zip((nx, ny, nz), layout):
        if v != orig or v < 2:
            raise _lib.RangeError("Grid dimensions must be integers of at least two cells.")
    b, nb = _mesh_array(body)
    s, ns = _mesh_array(supports)
    if b is None:
        b, nb = np.zeros(0, np.float32), 0
    out = C.c_void_p()
    L = _lib.load()
    _lib.check(L.pw_voxelize_opts(b.ctypes.data_as(C.c_void_p), nb,
                                  None if s is None else s.ctypes.data_as(C.c_void_p), ns,
                                  nx, ny, nz, int(bool(floor)), int(bool(link_fractions)), C.byref(out)), "voxelize")
    return _from_handle(out.value)


def grid_from_arrays(layout, geometry, boundary_cells) -> VoxelGrid:
    """A VoxelGrid from the reference's packed arrays, validated like
    validateGeometry (src/lbm/geometry-contract.ts:39-66)."""
    nx, ny, nz = (int(v) for v in layout)
    g = np.ascontiguousarray(geometry, np.uint32)
    b = np.ascontiguousarray(boundary_cells, np.uint32)
    out = C.c_void_p()
    _lib.check(_lib.load().pw_grid_from_host(nx, ny, nz, g.ctypes.data_as(C.c_void_p), g.size,
                                             b.ctypes.data_as(C.c_void_p) if b.size else None, b.size,
                                             C.byref(out)), "geometry")
    grid = _from_handle(out.value)
    grid._geometry = g.copy()
    grid._boundary = b.copy()
    return grid
