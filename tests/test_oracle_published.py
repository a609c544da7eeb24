"""The oracle against the reference's own published run: the laminar sphere
at tier S (docs/validation.md, sphere-re-100, 128x64x64, TRT, halfway walls,
f32 storage: Cd 1.1993, Cd voxel 1.2494, measured by the reference on WebGPU).
tests/golden/make_published_cases.py runs the same case on the binary32
restatement (6 flow-throughs, about five minutes) and records both; the
restatement matches every published digit, which pins it, and through it the
strict GPU build that equals it bit for bit, to the reference end to end."""
import json
import math
from pathlib import Path

GOLDEN = json.loads((Path(__file__).parent / "golden" / "published_cases.json").read_text())


def test_oracle_reproduces_the_published_sphere_drag():
    pub, ora = GOLDEN["published"], GOLDEN["oracle"]
    # the table gives four decimals
    assert abs(ora["cd"] - pub["cd"]) <= 5e-5
    assert abs(ora["cd_voxel"] - pub["cd_voxel"]) <= 5e-5
    # the two published coefficients imply the voxelized frontal area
    area = math.pi * 8 ** 2
    assert round(area * pub["cd"] / pub["cd_voxel"]) == ora["frontal_cells"] == 193
    assert ora["tau0"] == 0.524 and ora["steps"] == 15360 and ora["average_steps"] == 5120
