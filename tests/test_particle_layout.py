"""Particle seeding: restatement of tests/unit/render/particles.test.ts."""
import math
import struct

import numpy as np
import pytest

from pocketwind_gb300 import particle_layout as P
from pocketwind_gb300._lib import RangeError

LAYOUT = (32, 20, 20)
BMIN, BMAX = (8, 5, 5), (20, 15, 15)


def test_seed_region():
    assert P.seed_region(BMIN, BMAX, LAYOUT) == (3.5, 3.5, 16.5, 16.5)
    assert P.seed_region((8, 0, 0), (20, 20, 20), LAYOUT) == (1, 1, 18, 18)
    with pytest.raises(RangeError):
        P.seed_region(BMIN, BMAX, (4, 20, 20))
    with pytest.raises(RangeError):
        P.seed_region((0, 8, 8), (1, 7, 8), LAYOUT)
    with pytest.raises(RangeError):
        P.seed_region((0, 30, 30), (1, 40, 40), LAYOUT)


def test_reseed_rule():
    assert not P.particle_needs_reseed((2, 10, 10), 4000, LAYOUT, 1 << 4)
    assert not P.particle_needs_reseed((29.99, 10, 10), 0, LAYOUT, 0)
    assert P.particle_needs_reseed((30, 10, 10), 0, LAYOUT, 0)
    assert P.particle_needs_reseed((2, 10, 10), 4001, LAYOUT, 0)
    for kind in (1, 2, 3, 4):
        assert P.particle_needs_reseed((2, 10, 10), 1, LAYOUT, kind | (1 << 5))
    for pos in ((-1, 2, 2), (2, -1, 2), (2, 19, 2), (2, 2, -1), (2, 2, 19), (math.nan, 2, 2)):
        assert P.particle_needs_reseed(pos, 0, LAYOUT, 0)


def test_hash():
    assert P.particle_hash(0) == 0
    assert P.particle_hash(1) == 1753845952
    assert P.particle_hash(2) == 3507691905
    assert P.particle_hash(0xFFFFFFFF) == 1734902346


def test_seeds_only_fluid_inlet_nodes():
    geo = np.ones(32 * 20 * 20, np.uint32)
    geo[2 + 32 * (4 + 20 * 4)] = 1 << 4
    geo[2 + 32 * (5 + 20 * 4)] = 0
    data, region, fallback = P.particle_seeds(geo, LAYOUT, BMIN, BMAX, 4, 0)
    assert fallback == (2, 4, 4)
    assert data.nbytes == 128
    assert list(data.reshape(-1)) == [2, 4, 4, 0, 2, 4, 4, 0, 2, 4, 4, 0, 2, 4, 4, 0,
                                      2, 5, 4, 0, 2, 5, 4, 0, 2, 5, 4, 0, 2, 5, 4, 0]
    again, _, _ = P.particle_seeds(geo, LAYOUT, BMIN, BMAX, 4, 0)
    assert np.array_equal(again, data)
    other, _, _ = P.particle_seeds(geo, LAYOUT, BMIN, BMAX, 4, 1)
    assert not np.array_equal(other, data)


def test_seed_rejections():
    with pytest.raises(RangeError, match="no fluid inlet"):
        P.particle_seeds(np.ones(12800, np.uint32), LAYOUT, BMIN, BMAX, 1, 1)
    with pytest.raises(RangeError):
        P.particle_seeds(np.zeros(0, np.uint32), LAYOUT, BMIN, BMAX, 1, 1)
    geo = np.zeros(12800, np.uint32)
    for count in (0, 1.5, 65537):
        with pytest.raises(RangeError):
            P.particle_seeds(geo, LAYOUT, BMIN, BMAX, count, 1)
    for seed in (-1, 1.5, 2 ** 32):
        with pytest.raises(RangeError):
            P.particle_seeds(geo, LAYOUT, BMIN, BMAX, 1, seed)


def test_particle_params_packing():
    b = P.particle_params(LAYOUT, 1024, 0x12345678, 4.5, (3.5, 3.5, 16.5, 16.5), (2, 4, 5))
    assert len(b) == P.PARTICLE_PARAMS_BYTES
    assert list(struct.unpack("<5I", b[:20])) == [32, 20, 20, 1024, 0x12345678]
    assert list(struct.unpack("<11f", b[20:])) == [4.5, 0, 0, 3.5, 3.5, 16.5, 16.5, 4, 5, 0, 0]
    for steps in (-1, math.nan, math.inf, 1.7976931348623157e308):
        with pytest.raises(RangeError):
            P.particle_params(LAYOUT, 1, 1, steps, (1, 1, 2, 2), (2, 1, 1))


def test_sub_cell_cross_section():
    data, _, _ = P.particle_seeds(np.zeros(12800, np.uint32), LAYOUT, (8, 5.1, 6.1), (9, 5.2, 6.2), 1, 0)
    assert data[0, 0] == 2
    assert data[0, 1] == pytest.approx(5.085, abs=5e-6)
    assert data[0, 2] == pytest.approx(6.085, abs=5e-6)
    assert np.array_equal(data[0, 4:7], data[0, 0:3])


def test_float32_rounding_into_blocked_neighbour():
    geo = np.ones(12800, np.uint32)
    geo[2 + 32 * (5 + 20 * 6)] = 0
    with pytest.raises(RangeError, match="no fluid inlet"):
        P.particle_seeds(geo, LAYOUT, (8, 5.49999999, 6.1), (9, 5.5, 6.2), 1, 0)
