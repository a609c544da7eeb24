"""Pin the tracer and storage restatements to the reference's golden values.

* particles: tests/browser/particles.spec.ts:19-127 (golden trilinear Euler vector,
  displacement cap, age limit, respawn bounds and generations)
* storage:   tests/unit/precision/precision.test.ts:30-52 (quiet-flow f16 error with
  the 2^15 scale) and tests/browser/gpu-vs-cpu.spec.ts:638-653 (every stored
  equilibrium population within 1e-3 of its exact value)
"""
import numpy as np

from oracle import oracle as O
from tests.shapes import C, W


def _macros_linear():
    cells = 4096
    m = np.zeros((cells, 4), np.float32)
    for cell in range(cells):
        m[cell] = (2, (cell % 16) * 0.01, ((cell // 16) % 16) * 0.02, (cell // 256) * 0.03)
    return m.reshape(-1)


CS = (3.1, 3.1, 10.9, 10.9)  # seedRegion of body bounds [6,4,4]-[10,10,10] in 16^3


def _record(macros, steps, age=10, x=4.25, generation=0):
    p = np.array([x, 5.5, 6.75, age, x, 5.5, 6.75, generation], np.float32)
    flags = np.zeros(4096, np.uint32)
    return O.particles_update(p, macros, flags, (16, 16, 16), 7, steps, CS, (5.0, 5.0))


def test_particles_golden_vector():
    m = _macros_linear()
    got = _record(m, 2)
    for a, e in zip(got, [4.335, 5.72, 7.155, 11, 4.25, 5.5, 6.75, 0]):
        assert abs(a - e) < 5e-6
    const = np.tile(np.array([20, 3, 4, 0], np.float32), 4096)
    got = _record(const, 9)
    for a, e in zip(got, [4.85, 6.3, 6.75, 11, 4.25, 5.5, 6.75, 0]):
        assert abs(a - e) < 5e-6
    assert list(_record(const, 0)) == [4.25, 5.5, 6.75, 11, 4.25, 5.5, 6.75, 0]
    assert list(_record(const, 0, 3999)) == [4.25, 5.5, 6.75, 4000, 4.25, 5.5, 6.75, 0]
    expired = _record(const, 0, 4000)
    outlet = _record(const, 0, 10, 14)
    nxt = _record(const, 0, 4000, 4.25, 1)
    for r in (expired, outlet, nxt):
        assert r[0] == 2 and r[3] == 0 and list(r[4:7]) == list(r[0:3])
        assert all(3.1 <= c <= 10.9 for c in r[1:3])
    assert list(expired) == list(outlet)
    assert expired[7] == 1 and nxt[7] == 2
    assert list(nxt[1:3]) != list(expired[1:3])


def _shifted_eq(u):
    uu = np.dot(u, u)
    return np.array([W[i] * (3 * (C[i] @ u) + 4.5 * (C[i] @ u) ** 2 - 1.5 * uu) for i in range(19)])


def test_f16_quiet_flow_storage_error():
    exact = _shifted_eq(np.array([0.004, 0, 0]))
    for v in exact:
        stored = np.float16(np.float32(v * 32768)).astype(np.float64) / 32768
        assert abs(stored - v) / abs(v) < 1e-3
    smallest = np.abs(exact).min()
    assert smallest < 2 ** -14
    worst = max(abs(np.float16(v).astype(np.float64) - v) / abs(v) for v in exact)
    assert worst > 1e-3


def test_f16_hash_rounded_storage_error_bound():
    """Every dithered f16 code is one of the two neighbours of the value, so the
    stored population stays within 1e-3 (gpu-vs-cpu.spec.ts:638-653)."""
    for u in (0.004, 0.06):
        exact = _shifted_eq(np.array([u, 0, 0]))
        for i, v in enumerate(exact):
            for n in range(0, 32768, 997):
                code = O.encode_f16(np.float32(np.float32(v) * 32768), i, n)
                back = np.array([code], np.uint16).view(np.float16).astype(np.float64)[0] / 32768
                assert abs((back - v) / v) < 1e-3


def test_f16_codec_matches_numpy_rne():
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.normal(0, 1e-3, 4000), rng.normal(0, 100, 4000),
                           rng.uniform(-7e-5, 7e-5, 4000)]).astype(np.float32)
    lib = O.lib()
    got = np.array([lib.ow_f32_to_f16_rne(v) for v in vals], np.uint16)
    assert np.array_equal(got, vals.astype(np.float16).view(np.uint16))
    back = np.array([lib.ow_f16_to_f32(int(h)) for h in got], np.float32)
    assert np.array_equal(back, got.view(np.float16).astype(np.float32))
