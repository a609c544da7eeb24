"""GPU parity of the fused AA stream-collide against the CPU oracle.

Restates tests/browser/gpu-vs-cpu.spec.ts, force.spec.ts and nan-guard.spec.ts of
the reference on the CUDA path (through the C ABI):

* strict build (no fused multiply-add, reference expression order): every stored
  population, every macro and the drag equal the binary32 WGSL restatement bit for
  bit on the seeded 32^3 blob (TRT) -- the LES wall cell calls powf, whose last
  ulp may differ between CUDA and glibc, so REG+LES is held to the reference's
  1e-5 normalized error instead;
* fast build: normalized max error < 1e-5 (binary32 storage), < 2e-3 (f16, the
  reference's f16 bound) against the binary64 CpuSolver restatement, as the
  reference's browser test does (gpu-vs-cpu.spec.ts:17-19,186-190);
* drag: relative error < 1e-4 against the CPU reference (force.spec.ts:14).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.shapes import C, EQ, FLOOR, FLUID, NO_Q, SOLID, SUPPORT, W, blob_grid, grid_from_kinds

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4
LAYOUT = (32, 32, 32)
CELLS = 32 ** 3
F32_EPS = 2.0 ** -23


def _pw():
    from pocketwind_gb300 import geometry, solver
    return geometry, solver


def make_solver(geometry, boundary, layout=LAYOUT, tau0=0.8, u_in=0.06, les=False, op="trt",
                precision="f32", strict=False, ramp=0, kernel="auto", lateral="periodic", walls="bb"):
    G, S = _pw()
    grid = G.grid_from_arrays(layout, geometry, boundary)
    s = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=tau0, u_in=u_in, les=les, operator=op,
                                                         precision=precision, strict=strict, ramp_steps=ramp,
                                                         kernel=kernel, lateral=lateral, walls=walls))
    assert not isinstance(s, Exception)
    return s


def norm_err(actual, expected):
    """errorPeak + normalizedError of gpu-vs-cpu.spec.ts:166-190."""
    actual = np.asarray(actual, np.float64)
    expected = np.asarray(expected, np.float64)
    mag = np.abs(actual - expected)
    mag[~np.isfinite(actual) | ~np.isfinite(expected)] = np.inf
    return mag.max() / max(np.abs(expected).max(), F32_EPS)


CHECKPOINTS = [0, 1, 10, 50, 100]


@pytest.mark.parametrize("precision", ["f32", "f16", "bf16"])
def test_strict_blob_trt_is_bit_exact(precision):
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, precision=precision, strict=True)
    ref = O.Wgsl32(32, 32, 32, 0.8, 0.06, geometry, boundary, storage=precision, threads=THREADS)
    done = 0
    for cp in CHECKPOINTS:
        while done < cp:
            last = done == cp - 1
            gpu.step(1, last)
            ref.step(0.06, last)
            done += 1
        assert np.array_equal(gpu.populations_raw().view(np.uint32 if precision == "f32" else np.uint16),
                              ref.populations_raw().view(np.uint32 if precision == "f32" else np.uint16)), cp
        assert np.array_equal(gpu.macros().reshape(-1).view(np.uint32), ref.macros().view(np.uint32)), cp
        gpu.encode_force()
        f = gpu.read_force()
        assert f.step == cp
        assert np.allclose([f.fx, f.fy, f.fz], ref.force(), rtol=1e-12, atol=1e-15)


def test_strict_blob_reg_les_matches_binary32_reference():
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, les=True, op="reg", strict=True)
    ref = O.Wgsl32(32, 32, 32, 0.8, 0.06, geometry, boundary, les=True, op="reg", threads=THREADS)
    for _ in range(100):
        gpu.step(1, True)
        ref.step(0.06, True)
    assert norm_err(gpu.populations(), ref.populations()) < 1e-5
    assert norm_err(gpu.macros()[:, 1:], ref.macros().reshape(-1, 4)[:, 1:]) < 1e-5


CONFIGS = [("trt", False), ("reg", True)]


@pytest.mark.parametrize("op,les", CONFIGS)
def test_fast_blob_matches_fp64_reference(op, les):
    """gpu-vs-cpu.spec.ts:253-447: normalized max error < 1e-5 from step 0 to 100."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, les=les, op=op)
    cpu = O.Cpu64(LAYOUT, 0.8, operator=op, les=les, flags=geometry[:CELLS],
                  equilibrium_state=(1, (0.06, 0, 0)), threads=THREADS)
    done = 0
    for cp in CHECKPOINTS:
        while done < cp:
            gpu.step(1, done == cp - 1)
            cpu.step()
            done += 1
        if cp == 0:
            gpu.step(0, True)
        mac = gpu.macros().astype(np.float64)
        ref = cpu.macros()
        shifted = mac.copy()
        shifted[:, 0] -= 1
        ref_shift = ref.copy()
        ref_shift[:, 0] -= 1
        assert norm_err(gpu.populations(), cpu.populations) < 1e-5, cp
        assert norm_err(shifted[:, 0], ref_shift[:, 0]) < 1e-5, cp
        assert norm_err(shifted[:, 1:], ref_shift[:, 1:]) < 1e-5, cp
        gpu.encode_force()
        f = gpu.read_force()
        fr = cpu.momentum_exchange()
        scale = max(F32_EPS, np.abs(fr).max())
        assert np.abs(np.array([f.fx, f.fy, f.fz]) - fr).max() / scale < 1e-4, cp


def test_walls_rest_and_macros_preserved():
    """gpu-vs-cpu.spec.ts:193-215,398-410: wall cells keep rest, macros survive steps
    that do not write them."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary)
    gpu.step(1, True)
    after_one = gpu.macros().copy()
    gpu.step(98, False)
    assert np.array_equal(gpu.macros(), after_one)
    gpu.step(1, True)
    kinds = geometry[:CELLS] & 7
    walls = (kinds >= SOLID) & (kinds <= FLOOR)
    assert np.all(gpu.macros()[walls] == [1, 0, 0, 0])
    g = gpu.populations().reshape(19, CELLS)
    assert np.abs(g[:, walls]).max() == 0


@pytest.mark.parametrize("precision", ["f16", "bf16"])
@pytest.mark.parametrize("op,les", [("trt", False), ("reg", True)])
@pytest.mark.parametrize("centre", [(12, 12, 12), (12.3, 11.62, 12.41)])
def test_fast_16bit_within_reference_rounding_noise(precision, op, les, centre):
    """A voxelized sphere with EQ faces in 16-bit storage (the cell-pair kernel):
    after 16 steps the fast build is no further from the binary32 restatement
    in f32 storage than twice the restatement's own 16-bit storage (the
    reference's lowbias32 rounding) is.  The LES wall model's fall-backs switch
    on the tangential speed, so the reference's own f16 run differs from its
    f32 run by up to 16% of the largest population at the stagnation cells; the
    bound follows that noise instead of a fixed tolerance."""
    from pocketwind_gb300 import meshes
    from pocketwind_gb300.geometry import voxelize
    G, S = _pw()
    layout = (48, 24, 24)
    body = meshes.icosphere(centre, 4, 3)
    grid = voxelize(body, None, layout, False)
    ref_grid = O.voxelize(body.positions, None, layout, False, link_fractions=False)
    assert np.array_equal(grid.geometry, ref_grid.geometry)
    fast = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.56, u_in=0.05, les=les, operator=op,
                                                           precision=precision))
    ref32 = O.Wgsl32(*layout, 0.56, 0.05, ref_grid.geometry, ref_grid.boundary_cells, les=les, op=op)
    ref16 = O.Wgsl32(*layout, 0.56, 0.05, ref_grid.geometry, ref_grid.boundary_cells, les=les, op=op,
                     storage=precision)
    fast.step(16, True)
    for k in range(16):
        ref32.step(0.05, k == 15)
        ref16.step(0.05, k == 15)
    want = ref32.populations()
    err = norm_err(fast.populations(), want)
    ref_err = norm_err(ref16.populations(), want)
    assert np.isfinite(err) and err <= 2 * ref_err, (err, ref_err)
    fast.destroy()


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("precision,tol", [("f16", 2e-3), ("bf16", 2e-2)])
def test_16bit_storage_blob(precision, tol, strict):
    """gpu-vs-cpu.spec.ts:529-598: 16-bit storage within its bound after 100 steps.

    The density bound is a peak over 32768 cells of the dithered rounding noise.
    The strict build reproduces the reference's binary32 values and its hash, so
    its dither realization, and meets the reference's bound as the reference does.
    The fast build dithers with the same probabilities from another hash and from
    values that differ in the last bit, so it draws another realization of the
    same noise; across u_in perturbations of 1e-7 the density peak of either
    build spreads over 1.85e-3 .. 2.2e-3 at this size, so the fast build's
    density peak is held to 1.25 times the bound and its populations and
    velocities to the bound itself."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, precision=precision, strict=strict)
    cpu = O.Cpu64(LAYOUT, 0.8, flags=geometry[:CELLS], equilibrium_state=(1, (0.06, 0, 0)), threads=THREADS)
    gpu.step(100, True)
    cpu.step(100)
    assert norm_err(gpu.populations(), cpu.populations) < tol
    mac = gpu.macros().astype(np.float64)
    ref = cpu.macros()
    assert norm_err(mac[:, 0] - 1, ref[:, 0] - 1) < (tol if strict else 1.25 * tol)
    assert norm_err(mac[:, 1:], ref[:, 1:]) < tol


@pytest.mark.parametrize("u_in", [0.004, 0.06])
def test_f16_periodic_mass_drift(u_in):
    """gpu-vs-cpu.spec.ts:600-667: per-population storage error < 1e-3 and mean
    density drift < 2e-6 over 100 steps of a periodic uniform flow."""
    geometry = np.concatenate([np.zeros(CELLS, np.uint32), np.full(CELLS, NO_Q, np.uint32)])
    gpu = make_solver(geometry, np.zeros(0, np.uint32), u_in=u_in, precision="f16")
    exact = np.array([W[i] * (3 * C[i][0] * u_in + 4.5 * (C[i][0] * u_in) ** 2 - 1.5 * u_in ** 2) for i in range(19)])
    g0 = gpu.populations().reshape(19, CELLS).astype(np.float64)
    assert np.max(np.abs((g0 - exact[:, None]) / exact[:, None])) < 1e-3
    for _ in range(2):
        g = gpu.populations().astype(np.float64)
        assert abs(g.sum() / CELLS) < 2e-6
        gpu.step(100, False)


def test_force_known_answers():
    """cpu-solver.test.ts:136-154 and force.spec.ts:244-276 on the GPU: g*_1 = 0.01
    next to a SOLID cell gives Fx = 0.01 (2 g* halved by the mean with the rest
    state); SUPPORT and FLOOR links feel nothing."""
    for kind, expected in ((SOLID, 0.01), (SUPPORT, 0.0), (FLOOR, 0.0)):
        kinds = np.zeros(125, np.uint32)
        kinds[62] = kind
        geometry, boundary = grid_from_kinds((5, 5, 5), kinds)
        gpu = make_solver(geometry, boundary, layout=(5, 5, 5), u_in=0.0)
        gpu.encode_force()
        f = gpu.read_force()
        assert abs(f.fx) < 1e-15 and abs(f.fy) < 1e-15 and abs(f.fz) < 1e-15
        g = gpu.populations()
        g[1 * 125 + 61] = 0.01
        gpu.write_populations(g)
        gpu.encode_force()
        f = gpu.read_force()
        assert abs(f.fx - expected) < 1e-9 and abs(f.fy) < 1e-15 and abs(f.fz) < 1e-15
        gpu.step(1, True)
        mac = gpu.macros()[61]
        assert abs(mac[0] - 1.01) < 1e-6 and abs(mac[1] + 0.01 / 1.01) < 1e-6


def test_force_busy_slot_and_empty_boundary():
    """gpu-force.ts:174-210 and force.spec.ts:278-287."""
    geometry, boundary = grid_from_kinds((4, 4, 4), np.zeros(64, np.uint32))
    gpu = make_solver(geometry, boundary, layout=(4, 4, 4))
    assert gpu.read_force() == "busy"
    gpu.encode_force()
    gpu.step(8)
    gpu.encode_force()  # occupied slot: skipped, keeps its step stamp
    f = gpu.read_force()
    assert f.step == 0 and (f.fx, f.fy, f.fz) == (0, 0, 0)
    assert gpu.read_force() == "busy"
    gpu.encode_force()
    gpu.reset()  # drops the unread sample
    assert gpu.read_force() == "busy"


def test_period_two_oscillation_cancels_on_gpu():
    """cpu-solver.test.ts:158-168 through write-in of the latest state."""
    kinds = np.zeros(125, np.uint32)
    kinds[62] = SOLID
    geometry, boundary = grid_from_kinds((5, 5, 5), kinds)
    gpu = make_solver(geometry, boundary, layout=(5, 5, 5), u_in=0.0)
    g = gpu.populations()
    g[125 + 61] = 0.01
    gpu.write_populations(g)
    gpu.step(1)
    g = gpu.populations()
    g[125 + 61] = -0.01
    gpu.write_populations(g)
    gpu.encode_force()
    assert abs(gpu.read_force().fx) < 1e-15


def test_write_read_round_trip_and_totals():
    geometry, boundary = blob_grid("bb")
    for precision in ("f32", "f16"):
        gpu = make_solver(geometry, boundary, precision=precision)
        gpu.step(7, True)
        raw = gpu.populations_raw()
        gpu.write_populations_raw(raw)
        assert np.array_equal(gpu.populations_raw(), raw)
        g = gpu.populations().astype(np.float64).reshape(19, CELLS)
        kinds = geometry[:CELLS] & 7
        live = ~((kinds >= SOLID) & (kinds <= FLOOR))
        t = gpu.totals()
        assert abs(t[0] - g[:, live].sum()) < 1e-9
        for a in range(3):
            assert abs(t[1 + a] - (C[:, a][:, None] * g[:, live]).sum()) < 1e-9
        # the macros into a caller's buffer equal the ones into a fresh array
        buf = np.full((CELLS, 4), np.nan, np.float32)
        assert gpu.macros(out=buf) is buf and np.array_equal(buf, gpu.macros())
        for bad in (np.empty((CELLS, 4), np.float64), np.empty((CELLS, 3), np.float32),
                    np.empty((4, CELLS), np.float32).T):
            with pytest.raises(ValueError):
                gpu.macros(out=bad)


def test_ramp_matches_reference_schedule():
    """gpu-solver.ts:119-123,401-430: start at rest, ramp u_in linearly by
    rampFactor (its cases in tests/unit/stability.test.ts:155-171: 0 at step 0,
    step / ramp on the way, 1 from the ramp's end, 1 throughout without a ramp)."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, strict=True, ramp=20)
    ref = O.Wgsl32(32, 32, 32, 0.8, 0.06, geometry, boundary, threads=THREADS, u_in_init=0.0)
    for step in range(1, 31):
        gpu.step(1, True)
        ref.step(np.float32(0.06 * min(1.0, step / 20)), True)
    assert np.array_equal(gpu.populations_raw().view(np.uint32), ref.populations_raw().view(np.uint32))


def test_density_guard_and_nan_injection():
    """nan-guard.spec.ts:44-177: an injected NaN trips the guard on the next macro
    step; reset restores a stable state."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary)
    gpu.step(10, True)
    assert not gpu.guard_unstable()
    gpu.inject_nan()
    gpu.step(1, True)
    assert gpu.guard_unstable()
    gpu.reset()
    gpu.step(2, True)
    assert not gpu.guard_unstable()


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("precision", ["f16", "bf16", "f32"])
def test_nan_persists_until_the_guard_checks(precision, strict):
    """nan-guard.spec.ts:40-177 checks the density every few hundred steps, so a
    NaN must survive the steps between checks: stored as a NaN code (the
    reference's GPUs produce the quiet NaN 0x7fc00000, which its f16 rounding
    keeps), it spreads to the neighbours instead of being rounded to zero."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, precision=precision, strict=strict)
    gpu.step(4, True)
    gpu.inject_nan()
    gpu.step(6, False)
    assert np.isnan(gpu.populations()).sum() > 19
    gpu.step(1, True)
    assert gpu.guard_unstable()


def test_invalid_parameters_raise_range_error():
    G, S = _pw()
    geometry, boundary = blob_grid("bb")
    grid = G.grid_from_arrays(LAYOUT, geometry, boundary)
    with pytest.raises(S.RangeError):
        S.GpuSolver.create(LAYOUT, grid, S.SolverParams(tau0=0.5, u_in=0.05))
    with pytest.raises(S.RangeError):
        S.GpuSolver.create(LAYOUT, grid, S.SolverParams(tau0=0.8, u_in=float("nan")))
    with pytest.raises(S.RangeError):
        S.GpuSolver.create((32, 32, 16), grid, S.SolverParams(tau0=0.8, u_in=0.05))
    bad = geometry.copy()
    bad[100] ^= 1 << 10  # a wall bit that the pull neighbourhood does not justify
    with pytest.raises(S.RangeError):
        G.grid_from_arrays(LAYOUT, bad, boundary)


def _pair_equal(a, b, precision, exact=True):
    view = np.uint32 if precision == "f32" else np.uint16
    if exact:
        assert np.array_equal(a.populations_raw().view(view), b.populations_raw().view(view))
        assert np.array_equal(a.macros().view(np.uint32), b.macros().view(np.uint32))
    else:
        # The staged kernel rounds 16-bit codes with the reference's hash, the
        # cell kernel's plain cells with the fast build's; a code may then differ
        # by a unit of the stored precision, so 16-bit states are held to the
        # storage bound of the 16-bit comparison with binary64.
        tol = {"f32": 1e-5, "f16": 2e-3, "bf16": 2e-2}[precision]
        assert norm_err(a.populations(), b.populations()) < tol
        assert norm_err(a.macros()[:, 1:], b.macros()[:, 1:]) < tol
    a.encode_force()
    b.encode_force()
    fa, fb = a.read_force(), b.read_force()
    scale = max(F32_EPS, abs(fb.fx), abs(fb.fy), abs(fb.fz))
    tol = 1e-12 if exact else {"f32": 1e-4, "f16": 1e-3, "bf16": 8e-3}[precision]
    assert max(abs(fa.fx - fb.fx), abs(fa.fy - fb.fy), abs(fa.fz - fb.fz)) / scale < tol


STAGED_CASES = [(op, les, True) for op, les in CONFIGS] + [("trt", False, False)]


@pytest.mark.parametrize("precision", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("op,les,strict", STAGED_CASES)
def test_staged_rows_equal_cell_kernel_on_blob(precision, op, les, strict):
    """The TMA-staged kernel moves data differently but runs the same per-cell
    arithmetic: in the strict build the stored codes agree bit for bit with the
    one-cell-per-thread kernel (and so with the binary32 reference).  The fast
    build lets ptxas fuse multiply-adds per kernel, so there the two agree to the
    fast build's own tolerance; LES flows near the viscosity floor amplify those
    last-bit differences, so the fast comparison uses the laminar TRT case."""
    geometry, boundary = blob_grid("bb")
    a = make_solver(geometry, boundary, les=les, op=op, precision=precision, strict=strict, kernel="cell")
    b = make_solver(geometry, boundary, les=les, op=op, precision=precision, strict=strict, kernel="tile")
    for n in (1, 1, 6, 25):
        a.step(n, True)
        b.step(n, True)
        _pair_equal(a, b, precision, exact=strict)


@pytest.mark.parametrize("strict", [True])
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_staged_rows_equal_cell_kernel_on_vehicle(precision, strict):
    """Floor, EQ inlet/outlet planes, LES wall cells: 128 x 64 x 64 vehicle case."""
    from pocketwind_gb300 import meshes
    G, S = _pw()
    layout = (128, 64, 64)
    grid = G.voxelize(meshes.vehicle_case_mesh(128, 64), None, layout, True)
    mk = lambda k: S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.5 + 3 * 0.00625, u_in=0.05, les=True,
                                                                    operator="reg", precision=precision,
                                                                    strict=strict, kernel=k))
    a, b = mk("cell"), mk("tile")
    for n in (1, 3, 60, 200):
        a.step(n, True)
        b.step(n, True)
        _pair_equal(a, b, precision, exact=strict)


# ---------------------------------------------------------------- free-slip lateral faces
SLIP_CHECKPOINTS = [1, 10, 25, 50, 100]


@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_free_slip_strict_is_bit_exact(precision):
    """The free-slip option (no reference counterpart) against its binary32 restatement:
    the y and z faces reflect, wall links through the wrap are dropped, and the
    AA readout follows the reflected slots on odd steps."""
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, precision=precision, strict=True, lateral="free-slip")
    ref = O.Wgsl32(32, 32, 32, 0.8, 0.06, geometry, boundary, storage=precision, threads=THREADS,
                   lateral="free-slip")
    view = np.uint32 if precision == "f32" else np.uint16
    done = 0
    for cp in SLIP_CHECKPOINTS:
        while done < cp:
            last = done == cp - 1
            gpu.step(1, last)
            ref.step(0.06, last)
            done += 1
        assert np.array_equal(gpu.populations_raw().view(view), ref.populations_raw().view(view)), cp
        assert np.array_equal(gpu.macros().reshape(-1).view(np.uint32), ref.macros().view(np.uint32)), cp
        gpu.encode_force()
        f = gpu.read_force()
        assert np.allclose([f.fx, f.fy, f.fz], ref.force(), rtol=1e-12, atol=1e-15), cp


@pytest.mark.parametrize("op,les", CONFIGS)
def test_free_slip_fast_matches_fp64_reference(op, les):
    geometry, boundary = blob_grid("bb")
    gpu = make_solver(geometry, boundary, les=les, op=op, lateral="free-slip")
    cpu = O.Cpu64(LAYOUT, 0.8, operator=op, les=les, flags=geometry[:CELLS],
                  equilibrium_state=(1, (0.06, 0, 0)), threads=THREADS, lateral="free-slip")
    done = 0
    for cp in SLIP_CHECKPOINTS:
        while done < cp:
            gpu.step(1, done == cp - 1)
            cpu.step()
            done += 1
        assert norm_err(gpu.populations(), cpu.populations) < 1e-5, cp
        assert norm_err(gpu.macros()[:, 1:].astype(np.float64), cpu.macros()[:, 1:]) < 1e-5, cp


@pytest.mark.parametrize("precision,op,les", [("f16", "trt", False), ("f16", "reg", True), ("bf16", "trt", False),
                                               ("f32", "trt", False)])
def test_fast_step_is_deterministic(precision, op, les):
    """The fast build's step gives the same stored codes every time: its
    kernels run concurrently on two streams, and no cell's result may depend
    on their timing (an inflow or outflow cell's loads outside its row, which
    other cells rewrite during the step, once leaked into its equilibrium
    through rounding).  Four runs of the same voxelized sphere with EQ faces,
    60 steps each, are bit for bit equal."""
    from pocketwind_gb300 import meshes
    G, S = _pw()
    layout = (64, 32, 32)
    grid = G.voxelize(meshes.icosphere((16, 16, 16), 5, 3), None, layout, False)
    runs = []
    for _ in range(4):
        s = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.56, u_in=0.05, les=les, operator=op,
                                                            precision=precision))
        s.step(60, True)
        runs.append(s.populations_raw().view(np.uint8).copy())
        s.destroy()
    for r in runs[1:]:
        assert np.array_equal(r, runs[0])


def test_free_slip_write_read_round_trip_and_mass():
    """Write-in and readout follow the reflected slots in both layouts; a closed
    free-slip channel conserves mass."""
    geometry = np.concatenate([np.zeros(CELLS, np.uint32), np.full(CELLS, NO_Q, np.uint32)])
    gpu = make_solver(geometry, np.zeros(0, np.uint32), lateral="free-slip")
    rng = np.random.default_rng(5)
    for parity_steps in (3, 2):
        gpu.step(parity_steps)
        g = (rng.standard_normal(19 * CELLS) * 1e-3).astype(np.float32)
        gpu.write_populations(g)
        assert np.array_equal(gpu.populations(), g)
    m0 = gpu.totals()[0]
    gpu.step(40)
    assert abs(gpu.totals()[0] - m0) < 1e-9 * CELLS


def test_free_slip_rejects_the_staged_kernel():
    geometry, boundary = blob_grid("bb")
    G, S = _pw()
    grid = G.grid_from_arrays(LAYOUT, geometry, boundary)
    with pytest.raises(S.RangeError):
        S.GpuSolver.create(LAYOUT, grid, S.SolverParams(tau0=0.8, u_in=0.06, kernel="tile", lateral="free-slip"))


# ---------------------------------------------------------------- interpolated (Bouzidi) walls
@pytest.mark.parametrize("precision", ["f32", "f16"])
@pytest.mark.parametrize("op,les", [("trt", False), ("reg", True)])
def test_strict_blob_bouzidi_is_bit_exact(precision, op, les):
    """walls.wgsl:6-21 in the in-place kernel: the strict build equals the binary32
    restatement with A/B buffers bit for bit, populations, macros and the force of
    the two latest states, on the seeded blob with fractions on both sides of 1/2."""
    geometry, boundary = blob_grid("bouzidi")
    gpu = make_solver(geometry, boundary, precision=precision, strict=True, walls="bouzidi", op=op, les=les)
    ref = O.Wgsl32(32, 32, 32, 0.8, 0.06, geometry, boundary, storage=precision, walls="bouzidi", op=op, les=les,
                   threads=THREADS)
    view = np.uint32 if precision == "f32" else np.uint16
    done = 0
    for cp in CHECKPOINTS:
        while done < cp:
            last = done == cp - 1
            gpu.step(1, last)
            ref.step(0.06, last)
            done += 1
        assert np.array_equal(gpu.populations_raw().view(view), ref.populations_raw().view(view)), cp
        assert np.array_equal(gpu.macros().reshape(-1).view(np.uint32), ref.macros().view(np.uint32)), cp
        gpu.encode_force()
        f = gpu.read_force()
        assert f.step == cp
        assert np.allclose([f.fx, f.fy, f.fz], ref.force(), rtol=1e-12, atol=1e-15), cp


def test_fast_blob_bouzidi_matches_fp64_reference():
    """gpu-vs-cpu.spec.ts TRT + Bouzidi case: normalized max error < 1e-5 from step 0 to 100."""
    geometry, boundary = blob_grid("bouzidi")
    gpu = make_solver(geometry, boundary, walls="bouzidi")
    cpu = O.Cpu64(LAYOUT, 0.8, walls="bouzidi", flags=geometry, equilibrium_state=(1, (0.06, 0, 0)),
                  threads=THREADS)
    done = 0
    for cp in CHECKPOINTS:
        while done < cp:
            gpu.step(1, done == cp - 1)
            cpu.step()
            done += 1
        assert norm_err(gpu.populations(), cpu.populations) < 1e-5, cp
        if cp:
            assert norm_err(gpu.macros()[:, 1:], cpu.macros()[:, 1:]) < 1e-5, cp
        gpu.encode_force()
        f = gpu.read_force()
        fr = cpu.momentum_exchange()
        scale = max(F32_EPS, np.abs(fr).max())
        assert np.abs(np.array([f.fx, f.fy, f.fz]) - fr).max() / scale < 1e-4, cp


def test_bouzidi_differs_from_halfway_and_reset_repeats():
    geometry, boundary = blob_grid("bouzidi")
    bz = make_solver(geometry, boundary, walls="bouzidi", precision="f16")
    bb = make_solver(geometry, boundary, walls="bb", precision="f16")
    bz.step(30, True)
    bb.step(30, True)
    a = bz.populations()
    assert not np.array_equal(a, bb.populations())
    bz.reset()
    bz.step(30, True)
    assert np.array_equal(a, bz.populations())


def test_bouzidi_rejects_tile_and_free_slip():
    from pocketwind_gb300._lib import RangeError
    geometry, boundary = blob_grid("bouzidi")
    for kw in (dict(kernel="tile"), dict(lateral="free-slip")):
        with pytest.raises(RangeError):
            make_solver(geometry, boundary, walls="bouzidi", **kw)


def test_measured_sphere_bouzidi_drag_matches_fp64():
    """The whole row: measured link fractions from the GPU voxelizer feed the
    interpolated-wall solver; its drag follows the binary64 reference solver on
    the same geometry."""
    from pocketwind_gb300 import geometry as G, meshes, solver as S
    layout = (64, 32, 32)
    body = meshes.icosphere((16, 16, 16), 4.3, 3)
    grid = G.voxelize(body, None, layout, False, link_fractions=True)
    ref_grid = O.voxelize(body.positions, None, layout, False, link_fractions=True)
    geo = grid.geometry
    assert np.array_equal(geo, ref_grid.geometry)
    q = geo[2 * grid.cells:].view(np.float32)
    assert q.size and np.any(q < 0.5) and np.any(q > 0.5)
    nu = 0.05 * 8.6 / 40
    s = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.5 + 3 * nu, u_in=0.05, walls="bouzidi"))
    cpu = O.Cpu64(layout, 0.5 + 3 * nu, walls="bouzidi", flags=geo, equilibrium_state=(1, (0.05, 0, 0)),
                  threads=THREADS)
    for _ in range(4):
        s.step(50)
        for _ in range(50):
            cpu.step()
        s.encode_force()
        f = s.read_force()
        fr = cpu.momentum_exchange()
        assert abs(f.fx - fr[0]) < 1e-4 * abs(fr[0])
