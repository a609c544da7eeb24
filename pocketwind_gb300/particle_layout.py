"""Host-side seeding of the tracer particles (src/render/particle-layout.ts):
the seed region, the reseed rule the kernel applies, the seed hash, the initial
records and the fallback inlet node, and the advection parameters.

particle_seeds produces the records, cross-section and fallback that
tracers.Particles takes.
"""
from __future__ import annotations

import math
import struct
from typing import Sequence, Tuple

import numpy as np

from ._lib import RangeError

PARTICLE_BYTES = 32          # particle-layout.ts:6
PARTICLE_PARAMS_BYTES = 64   # particle-layout.ts:7
MAX_AGE_FRAMES = 4000        # particle-layout.ts:8
MAX_PARTICLES = 65536        # particle-layout.ts:9
FLUID = 0
SOLID = 1


def _js_round(v: float) -> int:
    return math.floor(v + 0.5)


def _safe_int(v) -> bool:
    return (isinstance(v, (int, float, np.integer, np.floating)) and not isinstance(v, bool)
            and math.isfinite(float(v)) and float(v) == int(v) and abs(int(v)) <= 2 ** 53 - 1)


def seed_region(bounds_min: Sequence[float], bounds_max: Sequence[float], layout) -> Tuple[float, float, float, float]:
    """seedRegion (particle-layout.ts:14-37): the body's y-z cross-section
    enlarged by 30% and clipped to interior cells, as (y0, z0, y1, z1)."""
    nx, ny, nz = layout
    ey = bounds_max[1] - bounds_min[1]
    ez = bounds_max[2] - bounds_min[2]
    region = (max(1, bounds_min[1] - ey * 0.15), max(1, bounds_min[2] - ez * 0.15),
              min(ny - 2, bounds_max[1] + ey * 0.15), min(nz - 2, bounds_max[2] + ez * 0.15))
    ok = (all(_safe_int(v) and v >= 5 for v in (nx, ny, nz))
          and all(math.isfinite(v) for v in (*bounds_min, *bounds_max))
          and ey > 0 and ez > 0 and region[0] < region[2] and region[1] < region[3])
    if not ok:
        raise RangeError("Particle seeds need a positive cross-section inside a grid of at least five cells per axis.")
    return region


def particle_needs_reseed(position: Sequence[float], age: float, layout, flag: int) -> bool:
    """particleNeedsReseed (particle-layout.ts:39-56): off the grid, past the
    outlet layer, older than MAX_AGE_FRAMES, or on a non-fluid node."""
    nx, ny, nz = layout
    x, y, z = (float(v) for v in position)
    return (not all(math.isfinite(v) for v in (x, y, z)) or x < 0 or x >= nx - 2 or y < 0 or y >= ny - 1
            or z < 0 or z >= nz - 1 or age > MAX_AGE_FRAMES or (int(flag) & 7) != FLUID)


def particle_hash(value: int) -> int:
    """particleHash (particle-layout.ts:58-63): a 32-bit xorshift-multiply mix."""
    r = int(value) & 0xFFFFFFFF
    r = ((r ^ (r >> 16)) * 0x7FEB352D) & 0xFFFFFFFF
    r = ((r ^ (r >> 15)) * 0x846CA68B) & 0xFFFFFFFF
    return (r ^ (r >> 16)) & 0xFFFFFFFF


def particle_seeds(geometry, layout, bounds_min, bounds_max, count: int, seed: int):
    """particleSeeds (particle-layout.ts:66-112): records (pos, age 0, prev =
    pos, 0) on fluid inlet nodes at x = 2 of the seed region, picked by
    particle_hash(id + seed); returns (records[count, 8], region, fallback)."""
    nx, ny, nz = layout
    region = seed_region(bounds_min, bounds_max, layout)
    geo = np.asarray(geometry, np.uint32).reshape(-1)
    if (not _safe_int(count) or count < 1 or count > MAX_PARTICLES or not _safe_int(seed) or seed < 0
            or seed > 0xFFFFFFFF or geo.size < nx * ny * nz):
        raise RangeError("Particle count, seed or geometry buffer is invalid.")
    f32 = lambda v: float(np.float32(v))
    inlet = []
    for z in range(_js_round(region[1]), _js_round(region[3]) + 1):
        for y in range(_js_round(region[0]), _js_round(region[2]) + 1):
            point = (2.0, f32(max(region[0], min(y, region[2]))), f32(max(region[1], min(z, region[3]))))
            i = 2 + nx * (_js_round(point[1]) + ny * _js_round(point[2]))
            flag = int(geo[i]) if 0 <= i < geo.size else SOLID
            if not particle_needs_reseed(point, 0, layout, flag):
                inlet.append(point)
    if not inlet:
        raise RangeError("The particle seed region has no fluid inlet cells.")
    fallback = inlet[0]
    data = np.zeros((int(count), 8), np.float32)
    for pid in range(int(count)):
        p = inlet[particle_hash((pid + int(seed)) & 0xFFFFFFFF) % len(inlet)]
        data[pid] = (*p, 0.0, *p, 0.0)
    return data, region, fallback


def particle_params(layout, count: int, seed: int, steps: float, region, fallback) -> bytes:
    """packParticleParams (particle-layout.ts:114-126): the 64-byte uniform."""
    with np.errstate(over="ignore", invalid="ignore"):
        s32 = np.float32(steps)  # Math.fround: values past the binary32 range become infinite
    if not (math.isfinite(float(s32)) and steps >= 0):
        raise RangeError("Particle advection needs non-negative finite solver steps.")
    nx, ny, nz = layout
    return struct.pack("<5I11f", nx, ny, nz, int(count), int(seed), float(steps), 0.0, 0.0, *region,
                       fallback[1], fallback[2], 0.0, 0.0)
