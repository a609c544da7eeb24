"""Batched stepping (pw_batch_*): members stepped together match the same
domains stepped alone; the autotuner keeps a working shape; misuse is refused.
The seeded case builder is checked on the CPU."""
import numpy as np
import pytest

from pocketwind_gb300 import cases


def test_splitmix64_known_answer():
    """splitmix64 seeded 0 (Steele, Lea and Flood): first outputs."""
    r = cases.SplitMix64(0)
    assert r.next() == 0xE220A8397B1DCDAF
    assert r.next() == 0x6E789E6AA1B965F4


def test_batch_tunnels_are_seeded_and_in_range():
    a, b = cases.batch_tunnels(64, 1), cases.batch_tunnels(64, 1)
    assert [t.layout for t in a] == [t.layout for t in b] and [t.re for t in a] == [t.re for t in b]
    assert {t.layout for t in a} <= set(cases.BATCH_SIZES)
    assert all(20 <= t.re <= 300 and t.tau0 >= 0.53 for t in a)
    assert {t.shape for t in a} == {"sphere", "ellipsoid", "box"}


def _norm_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 2.0 ** -23)


def _l2_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _make(tunnel, precision, lateral="periodic"):
    from pocketwind_gb300 import geometry, solver
    grid = geometry.voxelize(tunnel.body, None, tunnel.layout, False)
    return solver.GpuSolver.create(tunnel.layout, grid, solver.SolverParams(
        tau0=tunnel.tau0, u_in=0.05, precision=precision, lateral=lateral))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_batched_members_match_solo_runs(precision):
    from pocketwind_gb300.batch import Batch
    tunnels = cases.batch_tunnels(5, 3)
    solo = [_make(t, precision) for t in tunnels]
    together = [_make(t, precision) for t in tunnels]
    batch = Batch(together)
    for s in solo:
        s.step(57, True)
    batch.step(57, True)  # a captured 50-step graph, then 7 single launches
    for a, b in zip(together, solo):
        assert a.step_count == b.step_count == 57
        if precision == "f32":
            assert _norm_err(a.populations(), b.populations()) < 1e-5
            assert _norm_err(a.macros()[:, 1:], b.macros()[:, 1:]) < 1e-5
        else:
            # the batch kernel may fuse multiply-adds differently, and a last-bit
            # difference changes a code's dither: 16-bit states drift apart by a
            # few storage units per cell, so they are compared in relative L2
            assert _l2_err(a.populations(), b.populations()) < 5e-3
            assert _l2_err(a.macros()[:, 1:], b.macros()[:, 1:]) < 2e-3
        a.encode_force()
        b.encode_force()
        fa, fb = a.read_force(), b.read_force()
        assert fa.step == fb.step == 57
        assert abs(fa.fx - fb.fx) <= (1e-4 if precision == "f32" else 2e-3) * max(abs(fb.fx), 1e-6)
    batch.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_batched_members_match_the_reference_fp32_path(precision):
    """Members stepped through the batch's persistent launches against the
    oracle directly: the binary32 restatement of the reference's WGSL kernels
    (its A/B ping-pong, src/lbm/shaders/stream_collide.wgsl) run on each
    member's own voxel grid.  f32: populations within 1e-5 of the largest
    (the bound of the reference's GPU-vs-CPU browser test,
    tests/browser/gpu-vs-cpu.spec.ts) and drag within 1e-4.  f16: within
    twice the restatement's own f16 storage (lowbias32 rounding) distance
    from its f32 run."""
    from oracle import oracle as O
    from pocketwind_gb300 import geometry
    from pocketwind_gb300.batch import Batch
    tunnels = [t for t in cases.batch_tunnels(24, 9) if t.layout[0] <= 96][:3]
    assert len(tunnels) == 3
    members = [_make(t, precision) for t in tunnels]
    batch = Batch(members)
    steps = 57
    batch.step(steps, True)
    for t, m in zip(tunnels, members):
        grid = geometry.voxelize(t.body, None, t.layout, False)
        ref32 = O.Wgsl32(*t.layout, t.tau0, 0.05, grid.geometry, grid.boundary_cells, threads=4)
        for k in range(steps):
            ref32.step(0.05, k == steps - 1)
        want = ref32.populations()
        got = m.populations()
        if precision == "f32":
            assert _norm_err(got, want) < 1e-5
            m.encode_force()
            f = m.read_force()
            rf = ref32.force()
            assert abs(f.fx - rf[0]) <= 1e-4 * abs(rf[0])
        else:
            ref16 = O.Wgsl32(*t.layout, t.tau0, 0.05, grid.geometry, grid.boundary_cells, storage="f16", threads=4)
            for k in range(steps):
                ref16.step(0.05, k == steps - 1)
            assert _norm_err(got, want) <= 2 * _norm_err(ref16.populations(), want)
    batch.destroy()


@pytest.mark.gpu
def test_tuning_keeps_a_working_shape_and_reset_restarts():
    from pocketwind_gb300.batch import Batch
    tunnels = cases.batch_tunnels(4, 7)
    members = [_make(t, "f16") for t in tunnels]
    batch = Batch(members)
    t = batch.tune(4)
    assert t.candidates == 20 and t.rows_per_item in (8, 16, 32, 64) and t.blocks > 0 and t.ms_per_step > 0
    batch.reset()
    solo = [_make(x, "f16") for x in tunnels]
    batch.step(20, True)
    for s in solo:
        s.step(20, True)
    for a, b in zip(members, solo):
        assert _l2_err(a.macros()[:, 1:], b.macros()[:, 1:]) < 1e-3
    assert batch.time_steps(10) > 0
    batch.destroy()


@pytest.mark.gpu
def test_batch_refuses_mixed_or_misused_members():
    from pocketwind_gb300 import geometry, solver
    from pocketwind_gb300.batch import Batch
    t = cases.batch_tunnels(2, 5)
    a, b = _make(t[0], "f16"), _make(t[1], "f32")
    with pytest.raises(solver.RangeError):
        Batch([a, b])
    c = _make(t[1], "f16")
    grid = geometry.voxelize(t[0].body, None, t[0].layout, False)
    strict = solver.GpuSolver.create(t[0].layout, grid, solver.SolverParams(tau0=t[0].tau0, u_in=0.05,
                                                                             precision="f16", strict=True))
    with pytest.raises(solver.RangeError):
        Batch([a, strict])
    batch = Batch([a, c])
    a.step(1)
    with pytest.raises(solver.RangeError):
        batch.step(1)
    batch.destroy()
    # a member with a learned closure attached steps through the closure's own kernel
    from pocketwind_gb300.closure import Closure
    les = [solver.GpuSolver.create(t[k].layout, geometry.voxelize(t[k].body, None, t[k].layout, False),
                                   solver.SolverParams(tau0=t[k].tau0, u_in=0.05, precision="f16", les=True,
                                                       operator="reg")) for k in range(2)]
    net = Closure(1)
    net.attach(les[0])
    with pytest.raises(solver.RangeError):
        Batch(les)
    Closure.detach(les[0])
    Batch(les).destroy()
    net.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f16", "bf16"])
def test_floor_kernel_matches_the_general_path(precision):
    """A domain with a floor stepped alone runs its first fluid layer in the
    floor kernel (the LES wall cell of stream_collide.wgsl:18-80 in closed form
    for a flat floor); the same domain stepped in a batch takes those cells
    through the one-cell general path, which evaluates the wall cell in the
    reference's own order.  After 40 steps of the 64x32x32 vehicle (REG + LES
    + wall model) the two agree to the 16-bit storage's rounding (the bound of
    the batch's 16-bit comparison above), with the floor layer itself compared
    on its own."""
    from pocketwind_gb300 import solver
    from pocketwind_gb300.batch import Batch
    case = cases.vehicle_case(64)
    grid = case.grid()
    alone = solver.GpuSolver.create(case.layout, grid, case.params(precision))
    member = solver.GpuSolver.create(case.layout, grid, case.params(precision))
    batch = Batch([member])
    alone.step(40, True)
    batch.step(40, True)
    a, b = alone.macros().astype(np.float64), member.macros().astype(np.float64)
    nx, ny, nz = case.layout
    z = np.arange(nx * ny * nz) // (nx * ny)
    floor_layer = (z == 1) & ((grid.flags & 7) == 0)
    assert floor_layer.sum() > 0
    tol = 2e-3 if precision == "f16" else 1e-2  # bfloat16 keeps 8 bits
    for cells in (floor_layer, (grid.flags & 7) == 0):
        assert _l2_err(a[cells, 1:], b[cells, 1:]) < tol, cells.sum()
    alone.encode_force()
    member.encode_force()
    fa, fb = alone.read_force(), member.read_force()
    assert abs(fa.fx - fb.fx) <= tol * abs(fb.fx)
    batch.destroy()


@pytest.mark.gpu
def test_batch_step_is_deterministic():
    """A batch's two concurrent launches give the same stored codes every
    time: two batches of the same three tunnels, 60 steps each, are bit for
    bit equal member by member."""
    from pocketwind_gb300.batch import Batch
    tunnels = cases.batch_tunnels(3, 7)
    runs = []
    for _ in range(2):
        members = [_make(t, "f16") for t in tunnels]
        batch = Batch(members)
        batch.step(60, True)
        runs.append([m.populations_raw().view(np.uint8).copy() for m in members])
        batch.destroy()
        for m in members:
            m.destroy()
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)

