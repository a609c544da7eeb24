"""The benchmark's validation cases, built from their parameters.

* ``sphere_case``: the laminar sphere at Re 100 (the reference's
  ``laminarSphereCase``, src/validation/cases.ts:300-334: diameter nx/8 cells,
  u = 0.05, no floor, TRT) in a 96 x 48 x 48 tunnel with the sphere centred at
  x = 24, an icosphere of subdivision 4, viscosity set from Re (0.006; the
  reference's app clamps it at 0.01, units.ts:7,33), 4,000 steps with the drag
  averaged over steps 3,001-4,000, free-slip or periodic lateral faces;
* ``vehicle_case``: the rounded-nose bluff body with the 25 degree slant over a
  floor, Re 320 on its length, regularized collision with Smagorinsky LES and
  the wall model, at 128 x 64 x 64 (and scaled with nx).

``run_drag`` steps a ``GpuSolver`` and samples the drag every
``FORCE_EVERY_STEPS`` steps, as the reference's runners do.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

from . import forces, meshes
from .geometry import VoxelGrid, voxelize
from .solver import ForceSample, GpuSolver, SolverParams


@dataclass
class Case:
    name: str
    layout: tuple
    body: meshes.Mesh
    floor: bool
    tau0: float
    u_in: float
    operator: str
    les: bool
    lateral: str
    steps: int
    average_steps: int
    length_cells: float
    extra: dict = field(default_factory=dict)

    def grid(self) -> VoxelGrid:
        return voxelize(self.body, None, self.layout, self.floor)

    def params(self, precision: str = "f32", strict: bool = False) -> SolverParams:
        return SolverParams(tau0=self.tau0, u_in=self.u_in, les=self.les, operator=self.operator,
                            precision=precision, strict=strict, lateral=self.lateral)


def sphere_case(lateral: str = "free-slip", nx: int = 96, re: float = 100.0, subdivisions: int = 4) -> Case:
    ny = nz = nx // 2
    diameter = nx / 8
    u = forces.U_LU
    nu = u * diameter / re
    centre = (nx / 4, ny / 2, nz / 2)
    body = meshes.icosphere(centre, diameter / 2, subdivisions)
    return Case("sphere-re-%g" % re, (nx, ny, nz), body, False, 0.5 + 3 * nu, u, "trt", False, lateral,
                4000, 1000, diameter, {"re": re, "nu": nu, "diameter": diameter})


def vehicle_case(nx: int = 128, lateral: str = "periodic", steps: int = 20000) -> Case:
    scale = nx / 128
    ny = nz = nx // 2
    u = forces.U_LU
    length = 40 * scale
    nu = u * length / 320
    body = meshes.vehicle_case_mesh(nx, ny, scale)
    return Case("vehicle-re-320", (nx, ny, nz), body, True, 0.5 + 3 * nu, u, "reg", True, lateral,
                steps, 2 * forces.flow_through_steps(nx), length, {"re": 320.0, "nu": nu, "scale": scale})


def run_drag(solver: GpuSolver, steps: int, every: int = forces.FORCE_EVERY_STEPS) -> List[ForceSample]:
    """Step `steps` times, encoding and reading the drag every `every` steps."""
    samples = []
    done = 0
    while done < steps:
        k = min(every, steps - done)
        solver.step(k)
        done += k
        solver.encode_force()
        f = solver.read_force()
        if f != "busy":
            samples.append(f)
    return samples


def mean_drag(samples, steps: int, average_steps: int):
    return forces.averaged_forces(samples, steps, average_steps)
