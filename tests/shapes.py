"""Shared test inputs, restated from the reference's own test fixtures.

* ``box``         -- tests/unit/voxelize/fixtures.ts:5-20 (unit cube STL scaled to a box)
* ``blob_grid``   -- tests/browser/gpu-vs-cpu.spec.ts:54-116 (seeded 32^3 solid blob with
                     EQ slabs, one SUPPORT and one FLOOR cell, optional Bouzidi fractions)
* ``grid_from_kinds`` -- tests/browser/force.spec.ts:40-62 (pull masks from cell kinds)
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

from pocketwind_gb300.meshes import Mesh, _hypot

HERE = Path(__file__).resolve().parent
C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, -1, -1],
              [1, -1, 0], [-1, 1, 0], [1, 0, -1], [-1, 0, 1], [0, 1, -1], [0, -1, 1]])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
FLUID, SOLID, SUPPORT, FLOOR, EQ = 0, 1, 2, 3, 4
NO_Q = 0xFFFFFFFF


def opp(i):
    return 0 if i == 0 else (i + 1 if i % 2 == 1 else i - 1)


def _cube():
    d = json.loads((HERE / "golden" / "cube_binary.json").read_text())
    return np.array(d["positions"], np.float32)


def box(lo, hi, open_=False) -> Mesh:
    unit = _cube().astype(np.float64).reshape(-1, 3)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    p = (lo + unit * (hi - lo)).astype(np.float32)
    if open_:
        tris = p.reshape(-1, 9)
        fmax = np.float32(hi[0])
        keep = [t for t in tris if not (t[0] == fmax and t[3] == fmax and t[6] == fmax)]
        p = np.asarray(keep, np.float32)
    return Mesh(p.reshape(-1), p.size // 9)


def pull_mask(geometry, layout, cell):
    nx, ny, nz = layout
    x, y, z = cell % nx, (cell // nx) % ny, cell // (nx * ny)
    mask = 0
    for i in range(19):
        cx, cy, cz = C[i]
        src = (x - cx + nx) % nx + nx * (((y - cy + ny) % ny) + ny * ((z - cz + nz) % nz))
        k = int(geometry[src]) & 7
        if SOLID <= k <= FLOOR:
            mask |= 1 << (3 + i)
    return mask


def grid_from_kinds(layout, kinds):
    nx, ny, nz = layout
    cells = nx * ny * nz
    kinds = np.asarray(kinds, np.uint32)
    geometry = np.zeros(2 * cells, np.uint32)
    geometry[:cells] = kinds
    geometry[cells:] = NO_Q
    boundary = []
    for cell in range(cells):
        if kinds[cell] != FLUID:
            continue
        mask = pull_mask(kinds, layout, cell)
        geometry[cell] = mask
        if mask:
            boundary.append(cell)
    return geometry, np.array(boundary, np.uint32)


def _lcg(seed):
    return (seed * 1664525 + 1013904223) & 0xFFFFFFFF


def link_fractions(geometry, cells, seed):
    fractions = []
    geometry = geometry.copy()
    for cell in range(cells):
        flag = int(geometry[cell])
        if (flag & 7) != FLUID or (flag >> 3) == 0:
            continue
        geometry[cells + cell] = len(fractions)
        for i in range(1, 19):
            if flag & (1 << (3 + i)) == 0:
                continue
            seed = _lcg(seed)
            fractions.append(0.5 if len(fractions) % 7 == 0 else 0.05 + 0.95 * (seed / 2 ** 32))
    packed = np.concatenate([geometry, np.asarray(fractions, np.float32).view(np.uint32)])
    return packed


def blob_grid(walls="bb", layout=(32, 32, 32)):
    nx, ny, nz = layout
    cells = nx * ny * nz
    geometry = np.zeros(2 * cells, np.uint32)
    geometry[cells:] = NO_Q
    seed = 0x4A3B2C1D
    for cell in range(cells):
        x, y, z = cell % nx, (cell // nx) % ny, cell // (nx * ny)
        seed = _lcg(seed)
        radius = 5 + (seed / 2 ** 32) * 2
        if _hypot(x - 15.5, y - 15.5, z - 15.5) <= radius:
            geometry[cell] = SOLID
        if x < 2 or x >= nx - 2:
            geometry[cell] = EQ
    geometry[15 + nx * (15 + ny * 15)] = SUPPORT
    geometry[16 + nx * (15 + ny * 15)] = FLOOR
    kinds = geometry[:cells].copy()
    boundary = []
    for cell in range(cells):
        if kinds[cell] != FLUID:
            continue
        mask = pull_mask(kinds, layout, cell)
        geometry[cell] = mask
        if mask:
            boundary.append(cell)
    if walls == "bouzidi":
        geometry = link_fractions(geometry, cells, 0x1B873593)
    return geometry, np.array(boundary, np.uint32)
