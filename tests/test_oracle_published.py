"""The oracle against the reference's own published runs: the laminar sphere at
Re 100 (docs/validation.md, "Cases": sphere-re-100 with halfway walls and f32
storage, measured by the reference on WebGPU).  tests/golden/make_published_cases.py
runs the same cases on the binary32 restatement (6 flow-throughs each) and
records both; the restatement matches the published values within one unit of
their fourth decimal (TRT at tier S every digit) and the unrounded values to
1e-5, which pins it, and
through it the strict GPU build that equals it bit for bit, to the reference
end to end."""
import json
import math
from pathlib import Path

import pytest

CASES = json.loads((Path(__file__).parent / "golden" / "published_cases.json").read_text())["cases"]
TIERS = {"S": [128, 64, 64], "M": [192, 96, 96], "L": [256, 128, 128]}


@pytest.mark.parametrize("key", sorted(CASES))
def test_oracle_reproduces_the_published_sphere_drag(key):
    tier, _ = key.split(":")
    pub, ora = CASES[key]["published"], CASES[key]["oracle"]
    # the table's four decimals
    assert abs(ora["cd"] - pub["cd"]) <= 1e-4
    assert abs(ora["cd_voxel"] - pub["cd_voxel"]) <= 1e-4
    # the case's set-up: diameter nx / 8, nu = 0.05 D / 100, six flow-throughs, the last two averaged
    nx = TIERS[tier][0]
    assert ora["layout"] == TIERS[tier] and ora["diameter"] == nx // 8
    assert ora["tau0"] == 3 * (0.05 * (nx // 8) / 100) + 0.5
    assert ora["steps"] == 6 * math.ceil(nx / 0.05) and ora["average_steps"] == 2 * math.ceil(nx / 0.05)
    # the two published coefficients imply the voxelized frontal area
    area = math.pi * (nx // 16) ** 2
    assert round(area * pub["cd"] / pub["cd_voxel"]) == ora["frontal_cells"]


RESULTS = json.loads((Path(__file__).parent / "golden" / "published_results.json").read_text())


def _published(tier, operator):
    for row in RESULTS["laminar"]:
        if row["tier"] == tier and row["operator"] == operator:
            return row
    raise KeyError((tier, operator))


@pytest.mark.parametrize("key", sorted(CASES))
def test_oracle_against_the_full_precision_published_drag(key):
    """public/validation/results.json holds the reference's drag unrounded: the
    binary32 restatement agrees to within 1e-5 relative (measured 7e-7 with TRT
    and 5e-6 with REG at tier S; the reference ran on WebGPU, whose binary32
    operation order the restatement does not fix)."""
    tier, operator = key.split(":")
    row, ora = _published(tier, operator), CASES[key]["oracle"]
    assert row["steps"] == ora["steps"] and row["grid"]["nx"] == ora["layout"][0]
    assert abs(ora["cd"] / row["cd"] - 1) < 1e-5
    assert abs(ora["cd_voxel"] / row["cdVoxel"] - 1) < 1e-5


@pytest.mark.parametrize("operator", ["trt", "reg"])
def test_grid_convergence_reproduces_the_published_study(operator):
    """The reference's published grid convergence of the laminar sphere over
    tiers S, M and L (results.json "convergence": observed order, extrapolated
    Cd, fine-grid GCI; h = 1 / nx as src/validation/results.ts:213-216 takes it)
    from its own published drag, through reporting.grid_convergence."""
    from pocketwind_gb300 import reporting as R
    rows = [(1 / _published(t, operator)["grid"]["nx"], _published(t, operator)["cd"]) for t in ("S", "M", "L")]
    got = R.grid_convergence(rows)
    want = next(c for c in RESULTS["convergence"] if c["operator"] == operator)
    assert got.kind == want["kind"] == "monotone"
    assert math.isclose(got.order, want["order"], rel_tol=1e-9)
    assert math.isclose(got.extrapolated, want["extrapolated"], rel_tol=1e-12)
    assert math.isclose(got.gci_fine_pct, want["gciFinePct"], rel_tol=1e-9)


def test_oracle_grid_convergence_matches_the_published_study():
    """The restatement's own drag at tiers S, M and L (TRT) gives the reference's
    published convergence of the laminar sphere: observed order 1.3448 against
    1.3440, extrapolated Cd 1.17626 against 1.17624, GCI 0.958% against 0.959%."""
    from pocketwind_gb300 import reporting as R
    keys = ("S:trt", "M:trt", "L:trt")
    if not all(k in CASES for k in keys):
        pytest.skip("the fixture does not hold all three TRT tiers")
    got = R.grid_convergence([(1 / CASES[k]["oracle"]["layout"][0], CASES[k]["oracle"]["cd"]) for k in keys])
    want = next(c for c in RESULTS["convergence"] if c["operator"] == "trt")
    assert got.kind == "monotone"
    assert abs(got.order - want["order"]) < 5e-3
    assert abs(got.extrapolated - want["extrapolated"]) < 1e-4
    assert abs(got.gci_fine_pct - want["gciFinePct"]) < 1e-2
