"""Field export: the legacy VTK writer and the lattice-to-physical scaling of
src/io/vtk.ts:1-81 and src/io/field-export.ts:1-40.

``write_vtk`` formats host arrays exactly as writeVtk does (header lines, rho
and velocity as big-endian binary32, the newlines between and after the
blocks).  ``solver_vtk`` produces the same bytes for a solver's macros with the
body formatted on the GPU (pw_field_vtk_body), so a large field crosses PCIe
once, already in file order.
"""
from __future__ import annotations

import math
import re
from decimal import Decimal

import numpy as np

from ._lib import RangeError

U_LU = 0.05  # lattice inlet speed (src/lbm/units.ts:2)
_SAFE = 2 ** 53 - 1
_VECTORS = b"VECTORS velocity float\n"
# String.prototype.trim's WhiteSpace and LineTerminator code points
_JS_SPACE = ("\t\n\v\f\r \u00a0\u1680\u2000\u2001\u2002\u2003\u2004\u2005\u2006\u2007\u2008"
             "\u2009\u200a\u2028\u2029\u202f\u205f\u3000\ufeff")


def js_number(x) -> str:
    """ECMAScript Number::toString of a binary64 value, as a template literal
    prints it: shortest round-trip digits, plain notation for exponents
    -7 < e < 21, otherwise d.ddde+-x."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    if x == 0:
        return "0"
    if x < 0:
        return "-" + js_number(-x)
    sign, digits, exp = Decimal(repr(x)).normalize().as_tuple()
    s = "".join(str(d) for d in digits)
    k = len(s)
    n = exp + k  # x = 0.s * 10^n
    if k <= n <= 21:
        return s + "0" * (n - k)
    if 0 < n <= 21:
        return s[:n] + "." + s[n:]
    if -6 < n <= 0:
        return "0." + "0" * (-n) + s
    e = n - 1
    es = ("+" if e >= 0 else "-") + str(abs(e))
    return (s if k == 1 else s[0] + "." + s[1:]) + "e" + es


def _check_dimensions(nx, ny, nz) -> int:
    """checkDimensions (vtk.ts:14-21)."""
    for v in (nx, ny, nz):
        if isinstance(v, bool) or not isinstance(v, (int, float, np.integer, np.floating)):
            raise RangeError("Field dimensions must be positive integers.")
        if not (math.isfinite(float(v)) and float(v) == int(v) and 0 < int(v) <= _SAFE):
            raise RangeError("Field dimensions must be positive integers.")
    cells = int(nx) * int(ny) * int(nz)
    if cells > _SAFE:
        raise RangeError("The field is too large to address.")
    return cells


def _check_spacing(cell_size_m) -> None:
    if not (isinstance(cell_size_m, (int, float, np.integer, np.floating)) and math.isfinite(float(cell_size_m))
            and float(cell_size_m) > 0):
        raise RangeError("cellSizeM must be a positive finite number.")


def vtk_header(nx, ny, nz, cell_size_m) -> bytes:
    """The header lines of writeVtk (vtk.ts:42-56), ending with a newline."""
    cells = _check_dimensions(nx, ny, nz)
    _check_spacing(cell_size_m)
    s = js_number(cell_size_m)
    lines = [
        "# vtk DataFile Version 3.0",
        "PocketWind field",
        "BINARY",
        "DATASET STRUCTURED_POINTS",
        f"DIMENSIONS {js_number(nx)} {js_number(ny)} {js_number(nz)}",
        "ORIGIN 0 0 0",
        f"SPACING {s} {s} {s}",
        f"POINT_DATA {cells}",
        "SCALARS rho float 1",
        "LOOKUP_TABLE default",
        "",
    ]
    return "\n".join(lines).encode()


def write_vtk(nx, ny, nz, cell_size_m, rho, velocity) -> bytes:
    """writeVtk (vtk.ts:27-81): legacy binary STRUCTURED_POINTS with rho and
    interleaved velocity, big-endian binary32."""
    cells = _check_dimensions(nx, ny, nz)
    rho = np.asarray(rho, np.float32).reshape(-1)
    velocity = np.asarray(velocity, np.float32).reshape(-1)
    if rho.size != cells:
        raise RangeError(f"rho must hold {cells} values.")
    if velocity.size != 3 * cells:
        raise RangeError(f"velocity must hold {3 * cells} values.")
    _check_spacing(cell_size_m)
    return b"".join([vtk_header(nx, ny, nz, cell_size_m), rho.astype(">f4").tobytes(), b"\n", _VECTORS,
                     velocity.astype(">f4").tobytes(), b"\n"])


def _velocity_scale(speed_mps) -> float:
    if not (isinstance(speed_mps, (int, float, np.integer, np.floating)) and math.isfinite(float(speed_mps))
            and float(speed_mps) > 0):
        raise RangeError("speedMps must be a positive finite number.")
    return float(speed_mps) / U_LU


def lattice_to_field(velocity, speed_mps) -> np.ndarray:
    """latticeToField (field-export.ts:22-29): each binary32 lattice velocity
    times speedMps / U_LU in binary64, rounded back to binary32."""
    scale = _velocity_scale(speed_mps)
    return (np.asarray(velocity, np.float32).astype(np.float64) * scale).astype(np.float32)


def field_vtk_bytes(nx, ny, nz, cell_size_m, speed_mps, rho, velocity) -> bytes:
    """fieldVtkBytes (field-export.ts:31-33)."""
    return write_vtk(nx, ny, nz, cell_size_m, rho, lattice_to_field(velocity, speed_mps))


def field_file_name(name: str) -> str:
    """fieldFileName (field-export.ts:36-39)."""
    safe = re.sub(r'[\\/:*?"<>|]', "-", name).strip(_JS_SPACE)
    return f"{'untitled' if safe == '' else safe}-field.vtk"


def solver_vtk(solver, cell_size_m, speed_mps) -> bytes:
    """fieldVtkBytes of a solver's macros as last written: the header from the
    host, the body formatted on the GPU."""
    scale = _velocity_scale(speed_mps)
    nx, ny, nz = solver.layout
    header = vtk_header(nx, ny, nz, cell_size_m)
    return header + solver.field_vtk_body(scale)
