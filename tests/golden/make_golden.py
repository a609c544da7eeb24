"""Regenerate the golden fixtures in this directory from the reference checkout.

Run from the repository root in a container that has the reference mounted:
    python tests/golden/make_golden.py /path/to/pocketwind

cube_binary.json: the 12 facets of tests/fixtures/stl/cube-binary.stl, read the
way src/geometry/stl.ts:29-41 reads a binary STL (skip the 80-byte header and
4-byte count; per 50-byte record skip the normal, take nine little-endian
float32 coordinates).  tests/unit/voxelize/fixtures.ts:5-20 scales this unit
cube into the boxes the voxelizer tests use.

model_fixtures.json: the reference's mesh-import fixture files
(tests/fixtures/stl/*.stl, obj/*.obj, 3mf/*.3mf; each under 2 KB), base64, as
inputs for the importer tests (tests/unit/stl.test.ts, obj/obj.test.ts,
threemf/threemf.test.ts).

published_results.json: from the reference's public/validation/results.json,
the full-precision results of its laminar sphere cases (sphere-re-100: tier,
grid, operator, walls, storage, steps, Cd, Cd voxel), its grid-convergence
rows (observed order, extrapolated Cd, fine-grid GCI) and its verification
rows (Taylor-Green errors, order and decay; Poiseuille steps to convergence,
peak-speed and profile errors and force error), with the commit and date they
were measured at.

preset_geometry.json: the SHA-256 of the reference's published preset bodies
(public/validation/geometry/CHECKSUMS.txt: ahmed-25, cube, sphere and the
stilts, written by its scripts/export-geometry.ts as canonical binary STL), so
the preset generators can be checked byte for byte without the files.
"""
import base64
import json
import struct
import sys
from pathlib import Path


def read_binary_stl(path: Path):
    data = path.read_bytes()
    (count,) = struct.unpack_from("<I", data, 80)
    out = []
    for t in range(count):
        start = 84 + 50 * t + 12
        out.extend(struct.unpack_from("<9f", data, start))
    return count, out


def main():
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {Path(__file__).name} <path to the reference checkout> ...")
    ref = Path(sys.argv[1])
    count, positions = read_binary_stl(ref / "tests/fixtures/stl/cube-binary.stl")
    here = Path(__file__).resolve().parent
    (here / "cube_binary.json").write_text(json.dumps({
        "source": "tests/fixtures/stl/cube-binary.stl",
        "triangle_count": count,
        "positions": positions,
    }, indent=1) + "\n")
    print("wrote cube_binary.json with", count, "triangles")
    files = {}
    for sub in ("stl", "obj", "3mf"):
        for f in sorted((ref / "tests/fixtures" / sub).iterdir()):
            files[f"{sub}/{f.name}"] = base64.b64encode(f.read_bytes()).decode()
    (here / "model_fixtures.json").write_text(json.dumps({"source": "tests/fixtures/{stl,obj,3mf}",
                                                          "files": files}, indent=1) + "\n")
    print("wrote model_fixtures.json with", len(files), "files")
    sums = {}
    for line in (ref / "public/validation/geometry/CHECKSUMS.txt").read_text().splitlines():
        if line.strip():
            digest, name = line.split()
            sums[name] = digest
    (here / "preset_geometry.json").write_text(json.dumps({"source": "public/validation/geometry/CHECKSUMS.txt",
                                                           "sha256": sums}, indent=1) + "\n")
    print("wrote preset_geometry.json with", len(sums), "checksums")
    results = json.loads((ref / "public/validation/results.json").read_text())
    keep = ("case", "tier", "grid", "operator", "walls", "storage", "steps", "cd", "cdVoxel")
    laminar = [{k: r[k] for k in keep} for r in results["laminar"]]
    convergence = [{k: r[k] for k in ("case", "operator", "tiers", "kind", "order", "extrapolated", "gciFinePct")
                    if k in r} for r in results["convergence"] if r.get("case") == "sphere-re-100"]
    vkeep = ("case", "kind", "steps", "error", "observedOrder", "decayRelativeError", "errorPct", "profileErrorPct",
             "forceError", "tau0")
    verification = [{k: r.get(k) for k in vkeep} for r in results["verification"]]
    (here / "published_results.json").write_text(json.dumps({
        "source": "public/validation/results.json", "commit": results.get("commit"), "date": results.get("date"),
        "laminar": laminar, "convergence": convergence, "verification": verification}, indent=1) + "\n")
    print("wrote published_results.json with", len(laminar), "laminar rows")


if __name__ == "__main__":
    main()
