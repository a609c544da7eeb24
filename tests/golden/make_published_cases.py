"""Write published_cases.json: the reference's own published validation result
for the laminar sphere at tier S (docs/validation.md, "Cases" table:
sphere-re-100, S, 128x64x64, TRT, halfway walls, f32 storage), beside the same
case run on the binary32 restatement of the reference's kernels in oracle/.

Run from the repository root in a container that has the reference mounted
(about five minutes on eight cores):
    python tests/golden/make_published_cases.py /path/to/pocketwind

The case follows src/validation/cases.ts:300-337 and src/app/case-run.ts:
the sphere preset placed with a 16-cell diameter (nx / 8), the lattice
viscosity 0.05 * 16 / 100 (no floor), tau0 = 3 nu + 1/2, the inlet at 0.05
from an equilibrium start, a force sample after every 8 steps, 6 flow-throughs
(6 * ceil(128 / 0.05) steps) and the drag averaged over the last two.  Cd uses
the sphere's physical cross-section pi (D/2)^2 in cells, Cd voxel the voxelized
frontal cells.
"""
import json
import math
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import numpy as np  # noqa: E402

from oracle import oracle as O  # noqa: E402
from pocketwind_gb300 import meshes  # noqa: E402

LAYOUT = (128, 64, 64)
DIAMETER = LAYOUT[0] // 8
U = 0.05


def published_row(ref: Path):
    text = (ref / "docs/validation.md").read_text()
    for line in text.splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if cells[:3] == ["sphere-re-100", "laminar", "S"] and cells[5:8] == ["trt", "bb", "f32"]:
            return {"cd": float(cells[9]), "cd_voxel": float(cells[10]), "row": line.strip()}
    raise SystemExit("the sphere-re-100 S TRT row is missing from docs/validation.md")


def oracle_case():
    nu = U * DIAMETER / 100
    body, _ = meshes.place_mesh(meshes.preset_mesh("sphere"), *LAYOUT, DIAMETER, False)
    grid = O.voxelize(body.positions, None, LAYOUT, False, link_fractions=False)
    flow_through = math.ceil(LAYOUT[0] / U)
    steps, window = 6 * flow_through, 2 * flow_through
    solver = O.Wgsl32(*LAYOUT, 3 * nu + 0.5, U, grid.geometry, grid.boundary_cells, threads=os.cpu_count())
    drag = []
    for step in range(8, steps + 1, 8):
        for _ in range(8):
            solver.step(U, False)
        if step > steps - window:
            drag.append(float(solver.force()[0]))
    fx = float(np.mean(drag))
    area = math.pi * (DIAMETER / 2) ** 2
    return {"tau0": 3 * nu + 0.5, "steps": steps, "average_steps": window, "frontal_cells": int(grid.frontal_cells),
            "fx": fx, "cd": fx / (0.5 * U * U * area), "cd_voxel": fx / (0.5 * U * U * grid.frontal_cells)}


def main():
    ref = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    out = {"case": "sphere-re-100, tier S (128x64x64), TRT, halfway walls, f32 storage",
           "published": published_row(ref), "oracle": oracle_case()}
    (HERE / "published_cases.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
