"""Force reporting around the solver: physical units (src/forces/physical.ts),
reference areas (src/forces/reference-area.ts), grid convergence and the GCI
(src/forces/convergence.ts), the grid band (src/forces/grid-band.ts) and the
grid check that runs three refinements of one case (src/app/grid-check.ts).

The grid check keeps the reference's runner interface (one tier at a time,
each run disposed before the next, the previous run restored on every exit).
``gpu_grid_check`` is the GB300 runner: it creates the three tiers' domains
together and queues their steps on their own streams, so the three
refinements run concurrently on one GPU instead of one after another.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, List, Optional, Sequence, Tuple, Union

from ._lib import RangeError
from .forces import FORCE_EVERY_STEPS, U_LU, cd_per_lattice_force, flow_through_steps

RHO_AIR = 1.204  # standard air at 20 degrees Celsius, kg/m^3 (physical.ts:2)
AIR_DENSITY = RHO_AIR
NU_AIR = 1.5e-5  # m^2/s (src/lbm/units.ts:4)
NU_MIN_LU = 1e-2  # lattice viscosity floor (src/lbm/units.ts:7)


# ---------------------------------------------------------------- physical.ts
def _positive_finite(value, name: str) -> None:
    if not (isinstance(value, (int, float)) and math.isfinite(value) and value > 0):
        raise RangeError(f"{name} must be finite and positive.")


def cda_m2(cd: float, area_m2: float) -> float:
    """cdaM2 (physical.ts:12-18)."""
    if not (math.isfinite(cd) and cd >= 0):
        raise RangeError("Drag coefficient must be finite and non-negative.")
    _positive_finite(area_m2, "Reference area in square metres")
    return cd * area_m2


def drag_force_from_cda(cda: float, speed_mps: float, density_kgm3: float = RHO_AIR) -> float:
    """dragForceFromCda (physical.ts:21-28)."""
    if not (math.isfinite(cda) and cda >= 0):
        raise RangeError("CdA must be finite and non-negative.")
    _positive_finite(speed_mps, "Speed in metres per second")
    _positive_finite(density_kgm3, "Air density in kilograms per cubic metre")
    return 0.5 * density_kgm3 * speed_mps * speed_mps * cda


def drag_force_n(cd: float, area_m2: float, speed_mps: float, density_kgm3: float = RHO_AIR) -> float:
    """dragForceN (physical.ts:31-38)."""
    return drag_force_from_cda(cda_m2(cd, area_m2), speed_mps, density_kgm3)


def dynamic_pressure_pa(speed_mps: float, density_kgm3: float = RHO_AIR) -> float:
    """dynamicPressurePa (physical.ts:41-45)."""
    _positive_finite(speed_mps, "Speed in metres per second")
    _positive_finite(density_kgm3, "Air density in kilograms per cubic metre")
    return 0.5 * density_kgm3 * speed_mps * speed_mps


def cd_per_newton(area_m2: float, speed_mps: float, density_kgm3: float = RHO_AIR) -> float:
    """cdPerNewton (physical.ts:48-51)."""
    _positive_finite(area_m2, "Reference area in square metres")
    return 1 / (dynamic_pressure_pa(speed_mps, density_kgm3) * area_m2)


def physical_to_lattice(ref_length_cells: float, re: Optional[float] = None, speed_mps: Optional[float] = None,
                        ref_length_m: Optional[float] = None) -> Tuple[float, float]:
    """physicalToLattice (src/lbm/units.ts:22-37): (Re, lattice viscosity), the
    viscosity floored at NU_MIN_LU."""
    _positive_finite(ref_length_cells, "Reference length in cells")
    if re is None:
        _positive_finite(speed_mps, "Speed in metres per second")
        _positive_finite(ref_length_m, "Reference length in metres")
        re = speed_mps * ref_length_m / NU_AIR
    _positive_finite(re, "Reynolds number")
    nu = max(NU_MIN_LU, U_LU * ref_length_cells / re)
    _positive_finite(nu, "Lattice viscosity")
    return re, nu


# ---------------------------------------------------------------- reference-area.ts
def _safe_count(v) -> bool:
    """Number.isSafeInteger(v) && v >= 0."""
    return (isinstance(v, (int, float)) and not isinstance(v, bool) and math.isfinite(v) and float(v).is_integer()
            and 0 <= v <= 2 ** 53 - 1)


def reference_area_cells(preset_area_mm2: Optional[float], frontal_cells: int, cell_size_mm: float) -> float:
    """referenceAreaCells (reference-area.ts:11-25): the projected SOLID cells,
    or a preset's area in mm^2 over the cell area."""
    if preset_area_mm2 is None:
        if not _safe_count(frontal_cells):
            raise RangeError("Frontal cell count must be a non-negative safe integer.")
        return frontal_cells
    _positive_finite(preset_area_mm2, "Preset reference area in square millimetres")
    _positive_finite(cell_size_mm, "Cell size in millimetres")
    return preset_area_mm2 / (cell_size_mm * cell_size_mm)


def frontal_area_m2(frontal_cells: int, cell_size_m: float) -> float:
    """frontalAreaM2 (reference-area.ts:31-37)."""
    if not _safe_count(frontal_cells):
        raise RangeError("Frontal cell count must be a non-negative safe integer.")
    _positive_finite(cell_size_m, "Cell size in metres")
    return frontal_cells * cell_size_m * cell_size_m


# ---------------------------------------------------------------- convergence.ts
MAX_ROUNDS = 100
SETTLE_TOLERANCE = 1e-10
SAFETY_FACTOR = 1.25  # Celik et al. for an order observed on three grids


@dataclass(frozen=True)
class Monotone:
    order: float
    extrapolated: float
    gci_fine_pct: float
    kind: str = "monotone"


@dataclass(frozen=True)
class NotConverging:
    kind: str  # "oscillatory" | "divergent" | "insufficient"


GridConvergence = Union[Monotone, NotConverging]


def _sign(x: float) -> float:
    return (x > 0) - (x < 0)


def _observed_order(ratio: float, r21: float, r32: float, s: float) -> Optional[float]:
    """Fixed-point iteration for the order p of unequal refinement ratios
    (convergence.ts:12-21): p = |ln|e32/e21| + ln((r21^p - s)/(r32^p - s))| / ln r21."""
    order = 1.0
    for _ in range(MAX_ROUNDS):
        try:
            q = math.log((r21 ** order - s) / (r32 ** order - s))
        except (ValueError, ZeroDivisionError, OverflowError):
            return None
        nxt = abs(math.log(abs(ratio)) + q) / math.log(r21)
        if abs(nxt - order) < SETTLE_TOLERANCE:
            return nxt
        order = nxt
    return None


def grid_convergence(rows: Sequence[Tuple[float, float]]) -> GridConvergence:
    """gridConvergence (convergence.ts:28-49) of (h, value) rows: the three
    finest levels give the observed order, the Richardson limit and the
    fine-grid GCI in percent."""
    ordered = sorted(rows, key=lambda r: r[0])
    if len(ordered) < 3:
        return NotConverging("insufficient")
    (h1, f1), (h2, f2), (h3, f3) = ordered[:3]
    r21, r32 = h2 / h1, h3 / h2
    e21, e32 = f2 - f1, f3 - f2
    if e21 == 0 or e32 == 0:
        return NotConverging("insufficient")
    ratio = e32 / e21
    if ratio < 0:
        return NotConverging("oscillatory")
    if abs(e21) >= abs(e32):
        return NotConverging("divergent")
    order = _observed_order(ratio, r21, r32, _sign(ratio))
    if order is None or not math.isfinite(order):
        return NotConverging("divergent")
    factor = r21 ** order - 1
    extrapolated = (r21 ** order * f1 - f2) / factor
    gci = 100 * SAFETY_FACTOR * abs((f1 - f2) / f1) / factor
    return Monotone(order, extrapolated, gci)


# ---------------------------------------------------------------- grid-band.ts
@dataclass(frozen=True)
class Band:
    gci_pct: float
    extrapolated_cd: float
    kind: str = "band"


@dataclass(frozen=True)
class NoBand:
    reason: str
    kind: str = "no-band"


def grid_band(rows: Sequence[Tuple[float, float]]) -> Union[Band, NoBand]:
    """gridBand (grid-band.ts:13-22) of (h, Cd) rows."""
    for h, cd in rows:
        if not (math.isfinite(cd) and h > 0 and math.isfinite(h)):
            return NoBand("insufficient")
    r = grid_convergence(rows)
    if r.kind != "monotone":
        return NoBand(r.kind)
    return Band(r.gci_fine_pct, r.extrapolated)


# ---------------------------------------------------------------- grid-check.ts
TIERS = {"S": (128, 64, 64), "M": (192, 96, 96), "L": (256, 128, 128), "XL": (384, 192, 192)}  # layout.ts:7-11
GRID_CHECK_TIERS = ("S", "M", "L")
GRID_CHECK_FLOW_THROUGHS = 4
GRID_CHECK_L_LIMIT_S = 600
NO_BAND_TEXTS = {
    "oscillatory": "no grid band: the drag coefficient does not move steadily with grid size",
    "divergent": "no grid band: the drag coefficient changes more on finer grids",
    "insufficient": "no grid band: the three runs did not give a usable drag coefficient each",
}


def grid_check_length_cells(current_length_cells: float, current_nx: float, tier: str) -> int:
    """gridCheckLengthCells (grid-check.ts:68-73): the body keeps its share of
    the domain's length on every tier; halves round up as Math.round does."""
    if not (current_length_cells > 0) or not (current_nx > 0):
        raise RangeError("The run being checked needs a positive body length and grid length.")
    return max(1, math.floor(current_length_cells / current_nx * TIERS[tier][0] + 0.5))


def grid_check_steps(tier: str, run_flow_throughs: float) -> Tuple[int, int]:
    """gridCheckSteps (grid-check.ts:76-89): (total steps, averaged newest steps)."""
    if not (isinstance(run_flow_throughs, (int, float)) and math.isfinite(run_flow_throughs)
            and run_flow_throughs > 0):
        raise RangeError("The run length must be a positive number of flow-throughs.")
    ft = flow_through_steps(TIERS[tier][0])
    return math.ceil(run_flow_throughs * ft), math.ceil(run_flow_throughs / 2 * ft)


def predict_time_to_2t_s(tier_measured: str, ms_per_step: float, tier: str) -> float:
    """predictTimeTo2TS (src/lbm/tier-probe.ts:25-34): cell-ratio step cost over
    the target's two flow-throughs."""
    if not (math.isfinite(ms_per_step) and ms_per_step > 0):
        raise RangeError("Measured milliseconds per step must be finite and positive.")
    s, t = TIERS[tier_measured], TIERS[tier]
    ratio = (t[0] * t[1] * t[2]) / (s[0] * s[1] * s[2])
    return ms_per_step * ratio * (2 * t[0] / U_LU) / 1000


def predict_l_run_seconds(tier_measured: str, ms_per_step: float, run_flow_throughs: float) -> float:
    """predictLRunSeconds (grid-check.ts:92-97)."""
    return predict_time_to_2t_s(tier_measured, ms_per_step, "L") * run_flow_throughs / 2


def grid_check_availability(tier_measured: str, ms_per_step: float, tier_policy: str,
                            run_flow_throughs: float = GRID_CHECK_FLOW_THROUGHS) -> Tuple[str, Optional[str]]:
    """gridCheckAvailability (grid-check.ts:103-123): ("ready", None) or ("disabled", reason)."""
    if tier_policy == "s-only":
        return "disabled", "Check grid needs tiers M and L, and this GPU runs tier S only."
    seconds = predict_l_run_seconds(tier_measured, ms_per_step, run_flow_throughs)
    if seconds > GRID_CHECK_L_LIMIT_S:
        return "disabled", (f"Check grid is off: the tier L run is predicted at about "
                            f"{math.floor(seconds + 0.5)} s, above {GRID_CHECK_L_LIMIT_S} s.")
    return "ready", None


def mean_of_last(history: Sequence[Tuple[float, float]], average_steps: float) -> Optional[float]:
    """meanOfLast (grid-check.ts:126-135): mean Cd over the newest averageSteps."""
    if not history:
        return None
    last = history[-1][0]
    window = [cd for step, cd in history if step > last - average_steps]
    mean = sum(window) / len(window)
    return mean if math.isfinite(mean) else None


def grid_band_text(band: Union[Band, NoBand]) -> str:
    """gridBandText (grid-check.ts:203-206)."""
    if band.kind == "no-band":
        return NO_BAND_TEXTS[band.reason]
    return f"grid band ±{_to_fixed(band.gci_pct, 1)}% (extrapolated Cd {_to_fixed(band.extrapolated_cd, 3)})"


def _to_fixed(x: float, digits: int) -> str:
    """Number.prototype.toFixed: the exact binary value rounded half away from zero."""
    from decimal import ROUND_HALF_UP, Decimal
    return str(Decimal(x).quantize(Decimal(1).scaleb(-digits), rounding=ROUND_HALF_UP))


@dataclass(frozen=True)
class GridCheckRow:
    tier: str
    length_cells: int
    cd: Optional[float]


@dataclass(frozen=True)
class GridCheckDone:
    rows: Tuple[GridCheckRow, ...]
    band: Union[Band, NoBand]
    kind: str = "done"


@dataclass(frozen=True)
class GridCheckCancelled:
    kind: str = "cancelled"


class Cancelled(Exception):
    """Raised by a runner, or by ``cancelled()``, to stop a grid check."""


# A runner solves one tier with a body of the given length and returns
# (nx it used, history of (step, Cd) reaching the tier's total steps, dispose).
Runner = Callable[[str, int, int], Tuple[int, Sequence[Tuple[float, float]], Callable[[], None]]]


def run_grid_check(current_length_cells: float, current_nx: float, runner: Runner,
                   restore: Callable[[], None] = lambda: None,
                   run_flow_throughs: float = GRID_CHECK_FLOW_THROUGHS,
                   cancelled: Callable[[], bool] = lambda: False):
    """runGridCheck (grid-check.ts:171-196): S, M and L in turn, each disposed
    before the next starts, the previous run restored on every exit, then the
    band of the three means (h = 1 / body length in cells)."""
    rows: List[GridCheckRow] = []
    try:
        for tier in GRID_CHECK_TIERS:
            if cancelled():
                return GridCheckCancelled()
            length = grid_check_length_cells(current_length_cells, current_nx, tier)
            total, average = grid_check_steps(tier, run_flow_throughs)
            try:
                nx, history, dispose = runner(tier, length, total)
            except Cancelled:
                return GridCheckCancelled()
            except Exception:
                if cancelled():
                    return GridCheckCancelled()
                raise
            try:
                if nx != TIERS[tier][0]:
                    raise RuntimeError(f"The grid check asked for tier {tier} and the run used another grid.")
                if cancelled():
                    return GridCheckCancelled()
                rows.append(GridCheckRow(tier, length, mean_of_last(history, average)))
            finally:
                dispose()
    finally:
        restore()
    measured = [(1 / r.length_cells, r.cd) for r in rows if r.cd is not None]
    return GridCheckDone(tuple(rows), grid_band(measured))


# ---------------------------------------------------------------- GB300 runners
def _tier_solver(tier: str, length: int, body_mesh_for, re: float, precision: str, floor: bool):
    from . import geometry, solver as S
    layout = TIERS[tier]
    body, supports = body_mesh_for(length, layout)
    grid = geometry.voxelize(body, supports, layout, floor)
    frontal = grid.frontal_cells
    _, nu = physical_to_lattice(length, re=re)
    sv = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=3 * nu + 0.5, u_in=U_LU, les=True, operator="reg",
                                                         precision=precision))
    return sv, (cd_per_lattice_force(frontal) if frontal else float("nan"))


def gpu_tier_runner(body_mesh_for, re: float, precision: str = "f16", floor: bool = True,
                    every: int = FORCE_EVERY_STEPS) -> Runner:
    """A run_grid_check runner that solves one tier on the GPU: the body from
    ``body_mesh_for(length_cells, layout) -> (body, supports)``, viscosity from
    physical_to_lattice at Reynolds number ``re``, REG + LES, one Cd sample
    every ``every`` steps."""
    def run(tier, length, total):
        sv, scale = _tier_solver(tier, length, body_mesh_for, re, precision, floor)
        history = []
        try:
            while sv.step_count < total:
                sv.step(min(every, total - sv.step_count))
                sv.encode_force()
                f = sv.read_force()
                if f != "busy":
                    history.append((f.step, f.fx * scale))
        except BaseException:
            sv.destroy()
            raise
        return TIERS[tier][0], history, sv.destroy
    return run


def gpu_grid_check(body_mesh_for, current_length_cells: float, current_nx: float, re: float,
                   run_flow_throughs: float = GRID_CHECK_FLOW_THROUGHS, precision: str = "f16", floor: bool = True,
                   every: int = FORCE_EVERY_STEPS, tiers=GRID_CHECK_TIERS):
    """The grid check with the three tiers solved at once on one GPU.

    Each tier gets its own domain and stream (set up as gpu_tier_runner does);
    steps are queued to all tiers in rounds of ``every`` steps with one drag
    sample per round, so the GPU runs the tiers' kernels side by side rather
    than one tier after another.  The domains are independent, so every row
    equals the one-at-a-time run_grid_check bit for bit.  Returns the same
    GridCheckDone."""
    runs = []
    try:
        for tier in tiers:
            length = grid_check_length_cells(current_length_cells, current_nx, tier)
            total, average = grid_check_steps(tier, run_flow_throughs)
            sv, scale = _tier_solver(tier, length, body_mesh_for, re, precision, floor)
            runs.append(dict(tier=tier, length=length, total=total, average=average, solver=sv, scale=scale,
                             history=[]))
        while any(r["solver"].step_count < r["total"] for r in runs):
            live = [r for r in runs if r["solver"].step_count < r["total"]]
            for r in live:
                r["solver"].step(min(every, r["total"] - r["solver"].step_count))
                r["solver"].encode_force()
            for r in live:
                f = r["solver"].read_force()
                if f != "busy":
                    r["history"].append((f.step, f.fx * r["scale"]))
        rows = tuple(GridCheckRow(r["tier"], r["length"], mean_of_last(r["history"], r["average"])) for r in runs)
    finally:
        for r in runs:
            r["solver"].destroy()
    measured = [(1 / r.length_cells, r.cd) for r in rows if r.cd is not None]
    return GridCheckDone(rows, grid_band(measured))
