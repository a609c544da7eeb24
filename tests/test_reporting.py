"""Force reporting: restatements of tests/unit/convergence.test.ts,
tests/unit/forces/grid-band.test.ts, physical.test.ts, reference-area.test.ts
and tests/unit/app/grid-check.test.ts (plan, availability, mean, runner order,
cancel, refusal of a stepped-down grid, wording)."""
import math
import sys

import pytest

from pocketwind_gb300 import reporting as R
from pocketwind_gb300._lib import RangeError


def quadratic(h):
    return 1 + 0.5 * h ** 2


def monotone(rows):
    r = R.grid_convergence(rows)
    assert r.kind == "monotone", r
    return r


# ------------------------------------------------------------ convergence.test.ts
def test_order_two_from_four_grids():
    r = monotone([(h, quadratic(h)) for h in (1 / 384, 1 / 128, 1 / 256, 1 / 192)])
    assert abs(r.order - 2) < 0.01
    assert abs(r.extrapolated - 1) < 1e-6


def test_safety_factor_on_fine_index():
    r = monotone([(1, 1.5), (2, 3), (4, 9)])
    assert r.order == pytest.approx(2, abs=5e-10)
    assert r.extrapolated == pytest.approx(1, abs=5e-10)
    assert r.gci_fine_pct == pytest.approx(125 / 3, abs=5e-11)


def test_unequal_ratios():
    r = monotone([(1, 1.5), (2, 3), (6, 19)])
    assert abs(r.order - 2) < 1e-8 and abs(r.extrapolated - 1) < 1e-8


def test_coarser_levels_ignored():
    r = monotone([(1 / 8, quadratic(1 / 8)), (1 / 4, quadratic(1 / 4)), (1 / 2, quadratic(1 / 2)), (1, 42)])
    assert r.order == pytest.approx(2, abs=5e-10) and r.extrapolated == pytest.approx(1, abs=5e-10)


def test_not_converging_kinds():
    assert R.grid_convergence([(1, 1), (2, 2), (3, 1)]).kind == "oscillatory"
    assert R.grid_convergence([(1, 1), (2, 3), (3, 4)]).kind == "divergent"
    assert R.grid_convergence([(1, 1.5), (2, 3)]).kind == "insufficient"
    assert R.grid_convergence([(1, 1), (2, 1), (4, 2)]).kind == "insufficient"


# ------------------------------------------------------------ grid-band.test.ts
def test_band_from_monotone_rows():
    b = R.grid_band([(4, 9), (1, 1.5), (2, 3)])
    assert b.kind == "band"
    assert b.extrapolated_cd == pytest.approx(1, abs=5e-10)
    assert b.gci_pct == pytest.approx(125 / 3, abs=5e-10)


def test_no_band_reasons():
    assert R.grid_band([(1, 1), (2, 2), (3, 1)]) == R.NoBand("oscillatory")
    assert R.grid_band([(1, 1), (2, 3), (3, 4)]) == R.NoBand("divergent")
    assert R.grid_band([(1, 1.5), (2, 3)]) == R.NoBand("insufficient")
    assert R.grid_band([(1, 2), (2, 2), (4, 2)]) == R.NoBand("insufficient")
    assert R.grid_band([(1, math.nan), (2, 3), (4, 9)]) == R.NoBand("insufficient")
    assert R.grid_band([(0, 1), (2, 3), (4, 9)]) == R.NoBand("insufficient")


# ------------------------------------------------------------ physical.test.ts
def test_physical_units():
    assert R.RHO_AIR == 1.204 and R.AIR_DENSITY == R.RHO_AIR
    assert R.drag_force_n(0.3, 0.112, 40) == pytest.approx(0.5 * 1.204 * 1600 * 0.0336, abs=5e-13)
    area = R.cda_m2(0.3, 0.112)
    assert area == pytest.approx(0.0336, abs=5e-13)
    assert R.drag_force_n(0.3, 0.112, 40) == pytest.approx(R.drag_force_from_cda(area, 40), abs=5e-13)
    assert R.dynamic_pressure_pa(40) == pytest.approx(0.5 * 1.204 * 1600, abs=5e-13)
    assert R.drag_force_n(0.3, 0.112, 40) * R.cd_per_newton(0.112, 40) == pytest.approx(0.3, abs=5e-13)
    assert R.drag_force_n(0, 0.112, 40) == 0
    assert R.drag_force_n(0.3, 0.112, 40, 1.225) == pytest.approx(0.5 * 1.225 * 1600 * 0.0336, abs=5e-13)


@pytest.mark.parametrize("v", [-1, math.nan, math.inf])
def test_physical_rejects_bad_cd(v):
    with pytest.raises(RangeError):
        R.drag_force_n(v, 0.112, 40)
    with pytest.raises(RangeError):
        R.cda_m2(v, 0.112)
    with pytest.raises(RangeError):
        R.drag_force_from_cda(v, 40)


@pytest.mark.parametrize("v", [0, -1, math.nan, math.inf])
def test_physical_rejects_bad_area_speed(v):
    for call in (lambda: R.drag_force_n(0.3, v, 40), lambda: R.drag_force_n(0.3, 0.112, v),
                 lambda: R.cda_m2(0.3, v), lambda: R.cd_per_newton(v, 40), lambda: R.dynamic_pressure_pa(v)):
        with pytest.raises(RangeError):
            call()


# ------------------------------------------------------------ reference-area.test.ts
def test_reference_area():
    assert R.frontal_area_m2(100, 0.005) == 0.0025
    assert R.frontal_area_m2(0, 0.005) == 0
    assert R.reference_area_cells(112_000, 0, 10) == 1120
    assert R.reference_area_cells(None, 100, 0.005) == 100
    for v in (-1, 1.5, math.nan, math.inf):
        with pytest.raises(RangeError):
            R.frontal_area_m2(v, 0.005)
        with pytest.raises(RangeError):
            R.reference_area_cells(None, v, 10)
    for v in (0, -0.005, math.nan, math.inf):
        with pytest.raises(RangeError):
            R.frontal_area_m2(100, v)
        with pytest.raises(RangeError):
            R.reference_area_cells(112_000, 0, v)
    for v in (0, -1, math.nan, math.inf):
        with pytest.raises(RangeError):
            R.reference_area_cells(v, 0, 10)


def test_physical_to_lattice_floor():
    re, nu = R.physical_to_lattice(64, speed_mps=40, ref_length_m=1.0)
    assert re == pytest.approx(40 / 1.5e-5) and nu == R.NU_MIN_LU
    assert R.physical_to_lattice(12, re=20) == (20, 0.05 * 12 / 20)
    with pytest.raises(RangeError):
        R.physical_to_lattice(0, re=100)


# ------------------------------------------------------------ grid-check.test.ts
NX = {"S": 128, "M": 192, "L": 256}


def quadratic_cd(length_cells):
    return 1 + (1000 / length_cells) ** 2


def settled_history(tier, cd):
    total = math.ceil(0.5 * (NX[tier] / 0.05))
    return [(8, 100), (total - 16, cd), (total, cd)]


def test_plan():
    assert R.grid_check_length_cells(64, 128, "S") == 64
    assert R.grid_check_length_cells(64, 128, "M") == 96
    assert R.grid_check_length_cells(64, 128, "L") == 128
    assert R.grid_check_length_cells(51, 128, "M") == 77
    assert R.grid_check_length_cells(51, 128, "L") == 102
    with pytest.raises(RangeError):
        R.grid_check_length_cells(0, 128, "S")
    assert R.grid_check_steps("S", 4) == (10240, 5120)
    assert R.grid_check_steps("L", 0.5) == (2560, 1280)
    with pytest.raises(RangeError):
        R.grid_check_steps("S", 0)


def test_availability():
    assert R.predict_l_run_seconds("S", 1, 4) == pytest.approx(163.84, abs=5e-11)
    assert R.predict_l_run_seconds("S", 1, 0.5) == pytest.approx(20.48, abs=5e-11)
    assert R.grid_check_availability("S", 3.6, "s-m-l") == ("ready", None)
    kind, reason = R.grid_check_availability("S", 3.7, "s-m-l")
    assert kind == "disabled" and "above 600 s" in reason and "about 606 s" in reason
    assert R.grid_check_availability("S", 0.1, "s-only")[0] == "disabled"


def test_mean_of_last():
    assert R.mean_of_last([(100, 50), (700, 2), (1000, 4)], 400) == 3
    assert R.mean_of_last([], 400) is None
    assert R.mean_of_last([(8, math.nan)], 400) is None


def _fake_runner(log, cd_of=quadratic_cd):
    alive = [0]

    def run(tier, length, total):
        alive[0] += 1
        log.append(f"start {tier} {length} alive={alive[0]}")

        def dispose():
            alive[0] -= 1
            log.append(f"dispose {tier}")
        return NX[tier], settled_history(tier, cd_of(length)), dispose
    return run


def test_runs_in_order_and_restores():
    log = []
    res = R.run_grid_check(128, 128, _fake_runner(log), restore=lambda: log.append("restore"), run_flow_throughs=0.5)
    assert log == ["start S 128 alive=1", "dispose S", "start M 192 alive=1", "dispose M", "start L 256 alive=1",
                   "dispose L", "restore"]
    assert res.kind == "done"
    assert [r.length_cells for r in res.rows] == [128, 192, 256]
    assert [r.cd for r in res.rows] == [quadratic_cd(n) for n in (128, 192, 256)]
    assert res.band.kind == "band"
    assert res.band.extrapolated_cd == pytest.approx(1, abs=5e-7) and res.band.gci_pct > 0


def test_alternating_runs_give_no_band():
    cds = iter([3, 4, 3.5])
    res = R.run_grid_check(128, 128, _fake_runner([], lambda n: next(cds)), run_flow_throughs=0.5)
    assert res.kind == "done" and res.band == R.NoBand("oscillatory")


def test_cancel_between_runs():
    log = []
    flag = [False]

    def run(tier, length, total):
        log.append(f"start {tier}")
        if tier == "M":
            flag[0] = True
        return NX[tier], settled_history(tier, 2), lambda: log.append(f"dispose {tier}")
    res = R.run_grid_check(128, 128, run, restore=lambda: log.append("restore"), run_flow_throughs=0.5,
                           cancelled=lambda: flag[0])
    assert res.kind == "cancelled"
    assert log == ["start S", "dispose S", "start M", "dispose M", "restore"]


def test_runner_failing_after_cancel_is_cancelled():
    flag = [False]

    def run(tier, length, total):
        flag[0] = True
        raise RuntimeError("aborted")
    assert R.run_grid_check(128, 128, run, cancelled=lambda: flag[0]).kind == "cancelled"


def test_refuses_stepped_down_grid_and_restores():
    state = {"disposed": False, "restored": False}
    good = _fake_runner([])

    def run(tier, length, total):
        if tier == "S":
            return good(tier, length, total)

        def dispose():
            state["disposed"] = True
        return 128, [], dispose
    with pytest.raises(RuntimeError, match="another grid"):
        R.run_grid_check(128, 128, run, restore=lambda: state.update(restored=True), run_flow_throughs=0.5)
    assert state["disposed"] and state["restored"]


def test_band_wording():
    assert R.grid_band_text(R.Band(2.345, 0.3012)) == "grid band ±2.3% (extrapolated Cd 0.301)"
    texts = [R.grid_band_text(R.NoBand(r)) for r in ("oscillatory", "divergent", "insufficient")]
    assert texts == list(R.NO_BAND_TEXTS.values()) and len(set(texts)) == 3


# ------------------------------------------------------------ GPU
def _sphere_for(length, layout):
    from pocketwind_gb300 import meshes
    return meshes.place_mesh(meshes.preset_mesh("sphere"), *layout, length, False)


@pytest.mark.gpu
def test_concurrent_grid_check_equals_one_at_a_time():
    """The three tiers stepped side by side give the rows of the sequential
    check bit for bit, and every tier's Cd is a finite positive measurement."""
    conc = R.gpu_grid_check(_sphere_for, 16, 128, re=200.0, run_flow_throughs=0.25, floor=False)
    seq = R.run_grid_check(16, 128, R.gpu_tier_runner(_sphere_for, re=200.0, floor=False), run_flow_throughs=0.25)
    assert conc.rows == seq.rows and conc.band == seq.band
    assert [r.length_cells for r in conc.rows] == [16, 24, 32]
    for r in conc.rows:
        assert r.cd is not None and 0.1 < r.cd < 10


# ---------------------------------------------------------------- units.test.ts
def test_units_constants():
    """tests/unit/units/units.test.ts:11-15."""
    from pocketwind_gb300 import forces
    assert R.NU_AIR == 1.5e-5 and forces.U_LU == 0.05 and R.NU_MIN_LU == 1e-2


def test_physical_to_lattice_cases():
    """units.test.ts:17-51: nominal Re from metres, Reynolds similarity under
    refinement, a direct Re, and the viscosity floor at high Re."""
    re, nu = R.physical_to_lattice(102.4, speed_mps=40, ref_length_m=1.044)
    assert re == pytest.approx(2784000, abs=1e-8) and nu == R.NU_MIN_LU
    coarse = R.physical_to_lattice(20, speed_mps=5, ref_length_m=0.0001)
    fine = R.physical_to_lattice(40, speed_mps=5, ref_length_m=0.0001)
    assert fine[0] == coarse[0] and fine[1] == pytest.approx(2 * coarse[1], abs=1e-15)
    assert R.physical_to_lattice(20, re=100) == (100, 0.01)
    for re in (500000, 1000000, 1e12):
        assert R.physical_to_lattice(10, re=re) == (re, R.NU_MIN_LU)
    re, nu = R.physical_to_lattice(10, speed_mps=60, ref_length_m=1.044)
    assert re == pytest.approx(4176000, abs=1e-8) and nu == R.NU_MIN_LU


@pytest.mark.parametrize("value", [0, -1, math.nan, math.inf])
def test_physical_to_lattice_rejects_nonpositive_or_nonfinite_inputs(value):
    """units.test.ts:53-64."""
    for kwargs in (dict(ref_length_cells=20, re=value), dict(ref_length_cells=value, re=100),
                   dict(ref_length_cells=20, speed_mps=value, ref_length_m=1),
                   dict(ref_length_cells=20, speed_mps=40, ref_length_m=value)):
        with pytest.raises(RangeError):
            R.physical_to_lattice(**kwargs)


def test_physical_to_lattice_rejects_unrepresentable_derived_scales():
    """units.test.ts:66-73: an overflowing Re and an infinite viscosity."""
    with pytest.raises(RangeError):
        R.physical_to_lattice(20, speed_mps=sys.float_info.max, ref_length_m=2)
    with pytest.raises(RangeError):
        R.physical_to_lattice(20, re=5e-324)


def test_cd_per_lattice_force():
    """units.test.ts:76-86."""
    from pocketwind_gb300 import forces
    force = 0.5 * forces.U_LU * forces.U_LU * 432
    assert force * forces.cd_per_lattice_force(432) == pytest.approx(1, abs=1e-12)
    with pytest.raises(RangeError):
        forces.cd_per_lattice_force(0)
