"""The benchmark's accuracy figures as tests: the laminar sphere at Re 100
(96 x 48 x 48, FP32, TRT, 4,000 steps, drag averaged over steps 3,001-4,000)
and the 128 x 64 x 64 vehicle (REG + LES + wall model, floor) in each storage.

The vehicle is the benchmarked operator.  Its parity is pinned against the
reference's FP32 path (the binary32 restatement of its WGSL kernels,
``O.Wgsl32``) on the same voxel grid after 1,000 steps, at the tolerance the
benchmark states: velocity and density relative L2 below 1e-5, drag below
1e-4 (measured on GB300: 3.0e-6, 9.9e-8 and 9.0e-6; the strict build equals
the restatement exactly).  Beside it, the reference's own FP32 path is 2.5e-4
(velocity) from the binary64 CpuSolver on this case: a one-ulp change of one
population upstream of the body grows to 8e-6 of the velocity field within
200 steps, so this flow amplifies rounding, and 1e-5 is met only by following
the reference's FP32 path closely.  16-bit storage is held to the reference's
own 16-bit rounding of the same run (its f16 and bf16 storage against its own
f32): measured 6.1e-4 against 6.2e-4 (f16) and 3.4e-3 against 3.4e-3 (bf16)
in velocity.  BF16 cannot meet the 0.5% drag bar on this case: the
reference's own bf16 rounding misses it too (1.1% after 1,000 steps), because
bfloat16's 8-bit mantissa resolves the shifted populations (about 1e-2) only
to 4e-5, the size of the flow's disturbances near the body.
"""
import functools
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def _fp64_drag(case, grid, steps):
    cpu = O.Cpu64(case.layout, case.tau0, operator=case.operator, les=case.les, flags=grid.flags,
                  equilibrium_state=(1.0, (case.u_in, 0.0, 0.0)), threads=THREADS, lateral=case.lateral)
    out = []
    for k in range(8, steps + 1, 8):
        cpu.step(8)
        out.append((k, cpu.momentum_exchange()))
    return cpu, out


@pytest.mark.parametrize("lateral", ["free-slip", "periodic"])
def test_sphere_re100_drag_matches_fp64(lateral):
    from pocketwind_gb300 import cases, forces
    from pocketwind_gb300.solver import GpuSolver
    case = cases.sphere_case(lateral)
    grid = case.grid()
    s = GpuSolver.create(case.layout, grid, case.params("f32"))
    samples = cases.run_drag(s, case.steps)
    assert [x.step for x in samples] == list(range(8, case.steps + 1, 8))
    fx, fy, fz = cases.mean_drag(samples, case.steps, case.average_steps)
    _, ref = _fp64_drag(case, grid, case.steps)
    window = [f for k, f in ref if case.steps - case.average_steps < k <= case.steps]
    rfx = float(np.mean([f[0] for f in window]))
    assert abs(fx - rfx) / abs(rfx) < 1e-4
    # the sphere is symmetric: side forces stay small against the drag
    assert abs(fy) < 1e-3 * fx and abs(fz) < 1e-3 * fx
    cd = fx * forces.cd_per_lattice_force(grid.frontal_cells)
    assert 0.8 < cd < 2.0
    s.destroy()


def test_sphere_re100_fields_match_fp64_after_1000_steps():
    from pocketwind_gb300 import cases
    from pocketwind_gb300.solver import GpuSolver
    case = cases.sphere_case("free-slip")
    grid = case.grid()
    s = GpuSolver.create(case.layout, grid, case.params("f32"))
    s.step(1000, True)
    cpu = O.Cpu64(case.layout, case.tau0, flags=grid.flags, equilibrium_state=(1.0, (case.u_in, 0, 0)),
                  threads=THREADS, lateral=case.lateral)
    cpu.step(1000)
    m, r = s.macros().astype(np.float64), cpu.macros()
    fluid = (grid.flags & 7) == 0
    du = np.linalg.norm((m[:, 1:] - r[:, 1:])[fluid]) / np.linalg.norm(r[:, 1:][fluid])
    dr = np.linalg.norm((m[:, 0] - r[:, 0])[fluid]) / np.linalg.norm((r[:, 0] - 1)[fluid])
    assert du < 1e-5 and dr < 1e-4
    s.destroy()


VEHICLE_STEPS = 1000


def _field_errors(m, r, fluid):
    """Relative L2 over fluid cells of velocity, density, and the density
    deviation rho - 1, of macros m against r (n x 4: rho, ux, uy, uz)."""
    m = m.reshape(-1, 4).astype(np.float64)
    r = r.reshape(-1, 4).astype(np.float64)
    du = np.linalg.norm((m[:, 1:] - r[:, 1:])[fluid]) / np.linalg.norm(r[:, 1:][fluid])
    dr = np.linalg.norm((m[:, 0] - r[:, 0])[fluid]) / np.linalg.norm(r[:, 0][fluid])
    dd = np.linalg.norm((m[:, 0] - r[:, 0])[fluid]) / np.linalg.norm((r[:, 0] - 1.0)[fluid])
    return du, dr, dd


@functools.lru_cache(maxsize=1)
def _vehicle_references():
    """The 128 x 64 x 64 vehicle after VEHICLE_STEPS steps on the GPU voxelizer's
    grid: the reference's FP32 path in f32, f16 and bf16 storage (binary32
    restatement of its WGSL kernels, lowbias32 rounding) and the binary64
    CpuSolver restatement; macros and drag of each."""
    from pocketwind_gb300 import cases
    case = cases.vehicle_case(128)
    grid = case.grid()
    out = {"case": case, "grid": grid, "fluid": (grid.flags & 7) == 0}
    for storage in ("f32", "f16", "bf16"):
        w = O.Wgsl32(*case.layout, case.tau0, case.u_in, grid.geometry, grid.boundary_cells, les=True, op="reg",
                     storage=storage, threads=THREADS)
        for k in range(VEHICLE_STEPS):
            w.step(case.u_in, k == VEHICLE_STEPS - 1)
        out[storage] = (w.macros(), w.force())
    cpu = O.Cpu64(case.layout, case.tau0, operator="reg", les=True, flags=grid.flags,
                  equilibrium_state=(1.0, (case.u_in, 0.0, 0.0)), threads=THREADS)
    cpu.step(VEHICLE_STEPS)
    out["f64"] = (cpu.macros(), cpu.momentum_exchange())
    return out


def _gpu_vehicle(ref, precision, strict=False):
    from pocketwind_gb300.solver import GpuSolver
    case = ref["case"]
    s = GpuSolver.create(case.layout, ref["grid"], case.params(precision, strict=strict))
    s.step(VEHICLE_STEPS, True)
    m = s.macros()
    s.encode_force()
    f = s.read_force()
    s.destroy()
    return m, np.array([f.fx, f.fy, f.fz])


def test_vehicle_matches_reference_fp32_path():
    """Parity on the benchmarked operator (REG + Smagorinsky LES + the wall
    model, stream_collide.wgsl:8-136, collide-reg.wgsl:3-18), FP32 storage,
    1,000 steps, against the reference's FP32 path, as its GPU-vs-CPU browser
    test compares fields (tests/browser/gpu-vs-cpu.spec.ts:166-190): velocity
    and density within relative L2 1e-5, drag within 1e-4.  The strict build
    follows the restatement's expression order and matches it exactly here."""
    ref = _vehicle_references()
    fluid = ref["fluid"]
    w32, f32 = ref["f32"]
    m64, f64 = ref["f64"]
    fast, ff = _gpu_vehicle(ref, "f32")
    du, dr, dd = _field_errors(fast, w32, fluid)
    drag = abs(ff[0] - f32[0]) / abs(f32[0])
    assert du < 1e-5 and dr < 1e-5 and drag < 1e-4, (du, dr, drag)
    # the reference's own FP32 path against binary64 on the same case: the fast
    # build sits far closer to the reference's FP32 path than that path sits to
    # binary64 (velocity, and the density deviation rho - 1)
    ru, rr, rd = _field_errors(w32, m64, fluid)
    assert du < 0.1 * ru and dd < 0.25 * rd, (du, ru, dd, rd)
    strict, fs = _gpu_vehicle(ref, "f32", strict=True)
    su, sr, _ = _field_errors(strict, w32, fluid)
    # powf in the wall cells may differ from glibc's in the last ulp
    assert su < 1e-6 and sr < 1e-7 and abs(fs[0] - f32[0]) <= 1e-6 * abs(f32[0]), (su, sr)


@pytest.mark.parametrize("precision", ["f16", "bf16"])
def test_vehicle_16bit_storage_within_reference_rounding(precision):
    """16-bit storage on the benchmarked operator: the fast build's distance
    from the reference's FP32 path stays within 1.5 x the reference's own
    16-bit storage's distance from it (velocity and density), and its drag
    error against binary64 within 2 x the reference's own (each one dither
    realization)."""
    ref = _vehicle_references()
    fluid = ref["fluid"]
    w32, _ = ref["f32"]
    w16, f16 = ref[precision]
    _, f64 = ref["f64"]
    m, f = _gpu_vehicle(ref, precision)
    du, dr, _ = _field_errors(m, w32, fluid)
    ru, rr, _ = _field_errors(w16, w32, fluid)
    assert du <= 1.5 * ru and dr <= 1.5 * rr, (du, ru, dr, rr)
    drag, rdrag = abs(f[0] - f64[0]) / abs(f64[0]), abs(f16[0] - f64[0]) / abs(f64[0])
    assert drag <= max(2.0 * rdrag, 1e-3), (drag, rdrag)


def test_vehicle_f16_drag_unbiased_over_seeded_starts():
    """The f16 rounding adds noise but no bias to the drag: over eight seeded
    starts of the vehicle (1% velocity perturbations, 1,000 steps, drag
    averaged over the last 200), FP16 against FP32 from the same start has a
    relative drag error whose mean stays below 1e-4 and whose RMS below 3e-4
    (measured on GB300: mean 1.4e-5, RMS 6.1e-5, max 1.0e-4)."""
    from pocketwind_gb300 import cases, solver
    v = cases.vehicle_case(128)
    grid = v.grid()

    def drag(precision, seed):
        s = solver.GpuSolver.create(v.layout, grid, solver.SolverParams(tau0=v.tau0, u_in=0.05, les=True,
                                                                         operator="reg", precision=precision))
        cases.perturbed_start(s, grid, 0.05, 0.01, seed=seed)
        s.step(800)
        acc = 0.0
        for _ in range(25):
            s.step(8)
            s.encode_force()
            acc += s.read_force().fx
        s.destroy()
        return acc / 25

    err = np.array([drag("f16", k) / drag("f32", k) - 1.0 for k in range(1, 9)])
    assert abs(err.mean()) < 1e-4 and np.sqrt((err ** 2).mean()) < 3e-4, err


def test_vehicle_storage_errors_against_fp64():
    """Each storage against the binary64 CpuSolver restatement after 1,000
    steps: velocity and density relative L2 and drag.  The FP32 bounds sit at
    the reference's own FP32 distance from binary64 on this case (velocity
    2.5e-4, density 1.2e-6, drag 3e-5)."""
    ref = _vehicle_references()
    fluid = ref["fluid"]
    m64, fr = ref["f64"]
    bounds = {"f32": (5e-4, 1e-5, 1e-4), "f16": (2e-3, 1e-4, 2e-3), "bf16": (1e-2, 1e-3, 1.5e-2)}
    for precision, (bu, br, bd) in bounds.items():
        m, f = _gpu_vehicle(ref, precision)
        du, dr, _ = _field_errors(m, m64, fluid)
        dd = abs(f[0] - fr[0]) / abs(fr[0])
        assert du < bu and dr < br and dd < bd, (precision, du, dr, dd)


def _published_cases():
    import json
    from pathlib import Path
    return json.loads((Path(__file__).parent / "golden" / "published_cases.json").read_text())["cases"]


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("key", sorted(_published_cases()))
def test_published_sphere_case(key, strict):
    """The reference's published validation rows sphere-re-100 with halfway walls
    and f32 storage (docs/validation.md; case from src/validation/cases.ts:300-337
    and src/app/case-run.ts) on the GPU: the sphere preset at a diameter of
    nx / 8 cells, nu = 0.05 D / 100, a force sample every 8 steps, 6
    flow-throughs, the drag averaged over the last two.  The strict TRT build
    equals the binary32 restatement's drag (tests/golden/published_cases.json);
    the strict builds hold the published digits within 1e-4, the fast builds
    within 5e-4."""
    import math
    from pocketwind_gb300 import cases, forces, meshes
    from pocketwind_gb300.geometry import voxelize
    from pocketwind_gb300.solver import GpuSolver, SolverParams
    golden = _published_cases()[key]
    ora, pub = golden["oracle"], golden["published"]
    layout, diameter = tuple(ora["layout"]), ora["diameter"]
    operator = key.split(":")[1]
    body, _ = meshes.place_mesh(meshes.preset_mesh("sphere"), *layout, diameter, False)
    grid = voxelize(body, None, layout, False)
    assert grid.frontal_cells == ora["frontal_cells"]
    s = GpuSolver.create(layout, grid, SolverParams(tau0=ora["tau0"], u_in=0.05, operator=operator, strict=strict))
    steps, window = ora["steps"], ora["average_steps"]
    fx, _, _ = forces.averaged_forces(cases.run_drag(s, steps), steps, window)
    s.destroy()
    cd = fx / (0.5 * 0.05 ** 2 * math.pi * (diameter / 2) ** 2)
    cd_voxel = fx / (0.5 * 0.05 ** 2 * grid.frontal_cells)
    if strict and operator == "trt":  # the strict TRT step equals the restatement bit for bit
        assert abs(fx - ora["fx"]) <= 1e-9 * abs(fx)
    # the table's four decimals, and the reference's unrounded values
    # (public/validation/results.json): for the strict build 1e-5 relative with
    # TRT and 2e-5 with REG (the restatement: 1.4e-6 and 8e-6), 5e-4 for the
    # fast build
    tol = 1e-4 if strict else 5e-4
    assert abs(cd - pub["cd"]) <= tol
    assert abs(cd_voxel - pub["cd_voxel"]) <= tol
    import json
    from pathlib import Path
    results = json.loads((Path(__file__).parent / "golden" / "published_results.json").read_text())
    tier = key.split(":")[0]
    row = next(r for r in results["laminar"] if r["tier"] == tier and r["operator"] == operator)
    rel = (1e-5 if operator == "trt" else 2e-5) if strict else 5e-4
    assert abs(cd / row["cd"] - 1) < rel and abs(cd_voxel / row["cdVoxel"] - 1) < rel
