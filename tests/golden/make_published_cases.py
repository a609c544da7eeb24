"""Write published_cases.json: the reference's own published validation results
for the laminar sphere (docs/validation.md, "Cases" table: sphere-re-100 with
halfway walls and f32 storage, TRT and REG, tiers S = 128x64x64,
M = 192x96x96 and L = 256x128x128), beside the same cases run on the binary32 restatement of the
reference's kernels in oracle/.

Run from the repository root in a container that has the reference mounted
(about five minutes per S case, twenty-five per M case and eighty per L case
on eight cores;
existing rows of the file are kept, so cases can be added one at a time):
    python tests/golden/make_published_cases.py /path/to/pocketwind [S:trt,S:reg,M:trt,M:reg]

Each case follows src/validation/cases.ts:300-337 and src/app/case-run.ts:
the sphere preset placed with a diameter of nx / 8 cells, the lattice
viscosity 0.05 * diameter / 100 (no floor), tau0 = 3 nu + 1/2, LES off, the
inlet at 0.05 from an equilibrium start, a force sample after every 8 steps,
6 flow-throughs (6 * ceil(nx / 0.05) steps) and the drag averaged over the
last two.  Cd uses the sphere's physical cross-section pi (D/2)^2 in cells,
Cd voxel the voxelized frontal cells.
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

TIERS = {"S": (128, 64, 64), "M": (192, 96, 96), "L": (256, 128, 128)}  # gridFor, src/validation/cases.ts:135
U = 0.05


def published_row(ref: Path, tier: str, operator: str):
    text = (ref / "docs/validation.md").read_text()
    for line in text.splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if cells[:3] == ["sphere-re-100", "laminar", tier] and cells[5:8] == [operator, "bb", "f32"]:
            return {"cd": float(cells[9]), "cd_voxel": float(cells[10]), "row": line.strip()}
    raise SystemExit(f"the sphere-re-100 {tier} {operator} row is missing from docs/validation.md")


def oracle_case(tier: str, operator: str):
    layout = TIERS[tier]
    diameter = layout[0] // 8
    nu = U * diameter / 100
    body, _ = meshes.place_mesh(meshes.preset_mesh("sphere"), *layout, diameter, False)
    grid = O.voxelize(body.positions, None, layout, False, link_fractions=False)
    flow_through = math.ceil(layout[0] / U)
    steps, window = 6 * flow_through, 2 * flow_through
    solver = O.Wgsl32(*layout, 3 * nu + 0.5, U, grid.geometry, grid.boundary_cells, op=operator,
                      threads=os.cpu_count())
    drag = []
    for step in range(8, steps + 1, 8):
        for _ in range(8):
            solver.step(U, False)
        if step > steps - window:
            drag.append(float(solver.force()[0]))
    fx = float(np.mean(drag))
    area = math.pi * (diameter / 2) ** 2
    return {"layout": list(layout), "diameter": diameter, "tau0": 3 * nu + 0.5, "steps": steps,
            "average_steps": window, "frontal_cells": int(grid.frontal_cells), "fx": fx,
            "cd": fx / (0.5 * U * U * area), "cd_voxel": fx / (0.5 * U * U * grid.frontal_cells)}


def main():
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {Path(__file__).name} <path to the reference checkout> ...")
    ref = Path(sys.argv[1])
    wanted = (sys.argv[2] if len(sys.argv) > 2 else "S:trt").split(",")
    path = HERE / "published_cases.json"
    out = json.loads(path.read_text()) if path.exists() else {}
    out.setdefault("cases", {})
    for key in wanted:
        tier, operator = key.split(":")
        out["cases"][key] = {"case": f"sphere-re-100, tier {tier}, {operator.upper()}, halfway walls, f32 storage",
                             "published": published_row(ref, tier, operator),
                             "oracle": oracle_case(tier, operator)}
        path.write_text(json.dumps({"cases": out["cases"]}, indent=1) + "\n")
        print(key, json.dumps(out["cases"][key]["oracle"]), flush=True)


if __name__ == "__main__":
    main()
