"""Plate smoke layout: restatements of tests/unit/render/plate-layout.test.ts
(rake span, smoke parameters, physical time step, smoke front, dye ports)."""
import math
import struct

import numpy as np
import pytest

from pocketwind_gb300 import plate_layout as P
from pocketwind_gb300._lib import RangeError

GRID = (192, 96, 96)


def test_rake_span_inside_plate():
    z_top = 60.0
    low, high = P.rake_span(z_top, GRID[2])
    assert low > 1 and high <= z_top - 2 and high <= GRID[2] - 2
    assert P.rake_span(3.0, 96) == (1.5, 2.5)


def test_smoke_params_packing():
    b = P.smoke_params(GRID, 48, 7, True, 8, (1.5, 40))
    assert len(b) == P.SMOKE_PARAMS_BYTES
    assert list(struct.unpack("<8I", b[:32])) == [192, 96, 96, 48, P.THREADS, P.RING_SLOTS, 7, 1]
    assert list(struct.unpack("<4f", b[32:])) == [P.RAKE_X, 1.5, 40, 8]
    with pytest.raises(RangeError):
        P.smoke_params(GRID, 96, 0, False, 8, (1, 2))
    with pytest.raises(RangeError):
        P.smoke_params(GRID, 48, 2 ** 24, False, 8, (1, 2))


def test_seconds_per_step():
    assert P.seconds_per_step(1.044 / 96, 40, 0.05) == pytest.approx(1.359375e-5, abs=5e-13)
    with pytest.raises(RangeError):
        P.seconds_per_step(0, 40, 0.05)


def test_smoke_front():
    records = np.array([40.5, 3, 0, 0.9, 12, 7, 0, 0, 30, 9, 1024, 1, 55.25, 11, 0, 0.03], np.float32)
    assert P.smoke_front(records) == [(40.5, 3), (55.25, 11)]


def test_dye_ports_slanted_body():
    nx, ny, nz = 20, 3, 12
    flags = np.zeros(nx * ny * nz, np.uint32)
    plane = 1
    for z in range(2, 10):
        for x in range(4, 14 - max(0, z - 6) + 1):
            flags[x + nx * (plane + ny * z)] = 1
    ports = P.dye_ports(flags, (nx, ny, nz), plane, (2, 14))
    assert ports.size == P.PORTS * 2
    assert list(ports[0:2]) == [15, 4]
    assert list(ports[2:4]) == [13, 8]
    assert list(ports[4:6]) == [-1, -1]
    assert list(ports[6:8]) == [11, 10]
    assert list(ports[8:10]) == [15, 7]
    assert list(ports[10:12]) == [4, 1]


def test_dye_ports_smooth_body_separation():
    nx, ny, nz = 40, 3, 20
    flags = np.zeros(nx * ny * nz, np.uint32)
    plane = 1
    for z in range(nz):
        for x in range(nx):
            if ((x - 18) / 12) ** 2 + ((z - 9) / 5) ** 2 <= 1:
                flags[x + nx * (plane + ny * z)] = 1
    ports = P.dye_ports(flags, (nx, ny, nz), plane, (4, 14))
    x, z = int(ports[6]), int(ports[7])
    assert 22 < x < 30
    assert flags[x + nx * (plane + ny * (z - 1))] == 1
    lx, lz = int(ports[10]), int(ports[11])
    assert 22 < lx < 30
    assert flags[lx + nx * (plane + ny * (lz + 1))] == 1


def test_dye_ports_empty_plane():
    ports = P.dye_ports(np.zeros(10 * 3 * 8, np.uint32), (10, 3, 8), 1, (1.5, 5))
    assert np.all(ports == -1)
