"""Host-side layout of the plate smoke: the rake's height span, the dye ports
on the body, the advection parameters, the leading puffs and the physical time
step (src/render/plate-layout.ts).  The CSS fitting of the plate on a page
(fitPlate, plateToCss) is display code and is not restated; rake_span takes
the plate's top height in cells that fitPlate would give.

dye_ports feeds PlateSmoke(ports=...), smoke_params checks and packs what
PlateSmoke.advance sends to the kernel, smoke_front reads PlateSmoke.read().
"""
from __future__ import annotations

import math
import struct
from typing import List, Optional, Sequence, Tuple

import numpy as np

from ._lib import RangeError

RAKE_THREADS = 36          # plate-layout.ts:5
PORTS = 6                  # plate-layout.ts:15
BACK_PORTS = 3             # plate-layout.ts:16
THREADS = RAKE_THREADS + PORTS
RING_SLOTS = 8192          # plate-layout.ts:23
RELEASE_EVERY_FRAMES = 2   # plate-layout.ts:25
TEAR_CELLS = 3             # plate-layout.ts:27
SMOKE_PARAMS_BYTES = 48    # plate-layout.ts:28
RAKE_X = 2                 # plate-layout.ts:29
SEPARATION_DROP = 1.5      # plate-layout.ts:150-152
SEPARATION_RUN = 4
FLAT_UNDERSIDE = 0.25      # plate-layout.ts:154
SOLID = 1


def _js_round(v: float) -> int:
    """Math.round: halves round toward +infinity."""
    return math.floor(v + 0.5)


def rake_span(z_top: float, nz: int) -> Tuple[float, float]:
    """rakeSpan (plate-layout.ts:86-91): the lowest thread clears the floor, the
    highest stays a band below the top of the plate (z_top cells)."""
    low = 1.5
    return low, max(low + 1, min(nz - 2, z_top - 4.5))


def smoke_params(layout, plane: int, release: int, releasing: bool, steps: float,
                 rake: Sequence[float]) -> bytes:
    """packSmokeParams (plate-layout.ts:105-132): the 48-byte advection uniform,
    grid, plane, thread and slot counts, ring state (u32), then the rake x,
    its two heights and the step count (f32)."""
    nx, ny, nz = (int(v) for v in layout)
    ok = (isinstance(plane, (int, np.integer)) and 0 <= plane < ny
          and isinstance(release, (int, np.integer)) and 0 <= release < 2 ** 24 and steps >= 0)
    if not ok:
        raise RangeError("Smoke needs a plane inside the grid and a release index below 2^24.")
    return struct.pack("<8I4f", nx, ny, nz, int(plane), THREADS, RING_SLOTS, int(release), 1 if releasing else 0,
                       RAKE_X, float(rake[0]), float(rake[1]), float(steps))


def smoke_front(records) -> List[Tuple[float, float]]:
    """smokeFront (plate-layout.ts:139-147): (x, z) of every live puff that was
    the first released by its thread (release index 0)."""
    r = np.asarray(records, np.float32).reshape(-1)
    out = []
    for k in range(0, r.size - 3, 4):
        x, z, index, density = (float(v) for v in r[k:k + 4])
        if density > 0 and index == 0:
            out.append((x, z))
    return out


def seconds_per_step(cell_size_m: float, speed_mps: float, u_lu: float) -> float:
    """secondsPerStep (plate-layout.ts:227-232)."""
    if not (cell_size_m > 0 and speed_mps > 0 and u_lu > 0):
        raise RangeError("Cell size, speed and lattice speed must be positive.")
    return u_lu * cell_size_m / speed_mps


def dye_ports(flags, layout, plane: int, heights: Sequence[float]) -> np.ndarray:
    """dyePorts (plate-layout.ts:164-225): PORTS (x, z) cell pairs on the
    centre plane, -1 for a port with no body to sit on.  Three sit behind the
    base at evenly spaced heights in the rake's span; one above the separation
    line of the upper surface; one behind the top of the base; one under the
    nose of a flat underside, or below the separation line of a rounded one."""
    nx, ny, nz = (int(v) for v in layout)
    f = np.asarray(flags, np.uint32).reshape(-1)
    ports = np.full(PORTS * 2, -1.0, np.float32)

    def solid(x: int, z: int) -> bool:
        # the reference indexes the flat array, so x past the row reads on
        i = x + nx * (plane + ny * z)
        return 0 <= i < f.size and (int(f[i]) & 7) == SOLID

    xs = list(range(1, nx - 1))

    def rear_of(z: int) -> Optional[int]:
        for x in reversed(xs):
            if solid(x, z):
                return x
        return None

    rows = [z for z in range(1, nz - 1) if rear_of(z) is not None]

    def fluid(x: int, z: int) -> bool:
        return 1 <= x < nx - 1 and 1 <= z < nz - 1 and not solid(x, z)

    def place(slot: int, x: Optional[int], z: int) -> None:
        if x is not None and fluid(x, z):
            ports[2 * slot] = x
            ports[2 * slot + 1] = z

    low, high = heights
    for port in range(BACK_PORTS):
        z = _js_round(low + (high - low) * (port + 0.5) / BACK_PORTS)
        rear = rear_of(z) if 1 <= z < nz - 1 else None
        place(port, None if rear is None else rear + 1, z)
    if not rows:
        return ports
    top, bottom = rows[-1], rows[0]
    base = max(rear_of(z) or 0 for z in rows)
    base_top = [z for z in rows if rear_of(z) == base][-1] if any(rear_of(z) == base for z in rows) else top

    def crest_of(x: int) -> int:
        for z in reversed(rows):
            if solid(x, z):
                return z
        return 0

    crest = next((x for x in xs if crest_of(x) == top), base)
    separation = next((x for x in xs if crest <= x <= base and crest_of(x + 1) < crest_of(x)
                       and crest_of(x) - crest_of(x + SEPARATION_RUN) >= SEPARATION_DROP), None)
    place(BACK_PORTS, separation, 0 if separation is None else crest_of(separation) + 1)
    place(BACK_PORTS + 1, base + 1, base_top + 1)
    flat = [x for x in xs if solid(x, bottom)]
    front = next((x for x in xs if any(solid(x, z) for z in rows)), base)
    if len(flat) >= FLAT_UNDERSIDE * (base - front):
        place(BACK_PORTS + 2, flat[0] if flat else None, bottom - 1)
        return ports

    def keel_of(x: int) -> int:
        for z in rows:
            if solid(x, z):
                return z
        return nz

    keel = flat[-1] if flat else base
    lower = next((x for x in xs if keel <= x <= base and keel_of(x + 1) > keel_of(x)
                  and keel_of(x + SEPARATION_RUN) < nz
                  and keel_of(x + SEPARATION_RUN) - keel_of(x) >= SEPARATION_DROP), None)
    place(BACK_PORTS + 2, lower, 0 if lower is None else keel_of(lower) - 1)
    return ports
