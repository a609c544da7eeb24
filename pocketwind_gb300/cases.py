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
    walls: str = "bb"

    def grid(self) -> VoxelGrid:
        return voxelize(self.body, None, self.layout, self.floor, link_fractions=self.walls == "bouzidi")

    def params(self, precision: str = "f32", strict: bool = False) -> SolverParams:
        return SolverParams(tau0=self.tau0, u_in=self.u_in, les=self.les, operator=self.operator,
                            precision=precision, strict=strict, lateral=self.lateral, walls=self.walls)


def sphere_case(lateral: str = "free-slip", nx: int = 96, re: float = 100.0, subdivisions: int = 4,
                walls: str = "bb") -> Case:
    ny = nz = nx // 2
    diameter = nx / 8
    u = forces.U_LU
    nu = u * diameter / re
    centre = (nx / 4, ny / 2, nz / 2)
    body = meshes.icosphere(centre, diameter / 2, subdivisions)
    return Case("sphere-re-%g" % re, (nx, ny, nz), body, False, 0.5 + 3 * nu, u, "trt", False, lateral,
                4000, 1000, diameter, {"re": re, "nu": nu, "diameter": diameter}, walls)


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


# ---------------------------------------------------------------- batched tunnels
BATCH_SIZES = ((64, 32, 32), (96, 48, 48), (128, 64, 64), (192, 96, 96))
NU_MIN_LU = 1e-2  # the reference's lattice viscosity floor (src/lbm/units.ts:7,33)


class SplitMix64:
    """The splitmix64 generator (Steele, Lea and Flood, 2014): the seeded draws
    of the batched-tunnel case."""

    def __init__(self, seed: int):
        self.state = seed & 0xFFFFFFFFFFFFFFFF

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next() >> 11) * (1.0 / 9007199254740992.0))

    def choice(self, n: int) -> int:
        return min(n - 1, int(self.uniform() * n))


@dataclass
class Tunnel:
    layout: tuple
    shape: str
    body: meshes.Mesh
    re: float
    tau0: float
    length: float
    params_note: dict


def batch_tunnels(count: int = 64, seed: int = 1, u: float = forces.U_LU) -> List[Tunnel]:
    """Independent tunnels of uneven size and Reynolds number: sizes drawn
    uniformly from BATCH_SIZES, bodies a sphere, an ellipsoid (axis ratios
    U[1, 3]) or a box yawed U[0, 30] degrees, body length nx/8 centred at x =
    nx/4, Re U[20, 300] on that length, u = 0.05.  The lattice viscosity is
    max(0.01, u L / Re), the reference's floor, which keeps tau0 >= 0.53."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        nx, ny, nz = BATCH_SIZES[rng.choice(len(BATCH_SIZES))]
        kind = ("sphere", "ellipsoid", "box")[rng.choice(3)]
        re = rng.uniform(20.0, 300.0)
        length = nx / 8
        centre = (nx / 4, ny / 2, nz / 2)
        note = {}
        if kind == "sphere":
            body = meshes.icosphere(centre, length / 2, 3)
        elif kind == "ellipsoid":
            ry, rz = rng.uniform(1.0, 3.0), rng.uniform(1.0, 3.0)
            body = meshes.ellipsoid(centre, (length / 2, length / 2 / ry, length / 2 / rz), 3)
            note = {"axis_ratios": (ry, rz)}
        else:
            yaw = rng.uniform(0.0, 30.0)
            body = meshes.yawed_box(centre, (length, length / 2, length / 2), yaw)
            note = {"yaw_deg": yaw}
        nu = max(NU_MIN_LU, u * length / re)
        out.append(Tunnel((nx, ny, nz), kind, body, re, 0.5 + 3 * nu, length, note))
    return out


# ---------------------------------------------------------------- closure data
def perturbed_start(solver: GpuSolver, grid: VoxelGrid, u_in: float, amplitude: float = 0.01, seed: int = 1) -> None:
    """Start a domain from equilibrium at rho 1 and the inflow velocity with a
    seeded uniform perturbation of `amplitude` * u_in on each component of each
    fluid cell (walls at rest): the seeded inflow perturbations of the closure's
    training runs."""
    import numpy as np
    cells = grid.nx * grid.ny * grid.nz
    rng = np.random.default_rng(seed)
    u = np.empty((3, cells), np.float64)
    u[0] = u_in
    u[1:] = 0.0
    u += amplitude * u_in * rng.uniform(-1.0, 1.0, (3, cells))
    kind = grid.flags & 7
    walls = (kind >= 1) & (kind <= 3)
    u[:, walls] = 0.0
    cx = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
    cy = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
    cz = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    uu = (u * u).sum(0)
    g = np.empty((19, cells), np.float32)
    for i in range(19):
        cu = cx[i] * u[0] + cy[i] * u[1] + cz[i] * u[2]
        g[i] = w[i] * (3 * cu + 4.5 * cu * cu - 1.5 * uu)
    g[:, walls] = 0.0
    solver.write_populations(g.reshape(-1))
