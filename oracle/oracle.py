"""ctypes wrapper over the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module, and only as the checker: the shipped library never calls it.  The C
sources it wraps restate the reference (intesarjawad/pocketwind):

* ``Wgsl32``  -- src/lbm/shaders/*.wgsl in binary32 (lbm_f32.c)
* ``Cpu64``   -- src/lbm/reference/cpu-solver.ts + collision.ts in binary64 (lbm_f64.c)
* ``voxelize``/``build_wall_links``/``nearest_link_hit`` -- src/geometry (geometry.c)
* ``particles_update``/``plate_smoke``/``streaks`` -- src/render/shaders (tracers.c)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import build as _build

_lib = None

OPERATORS = {"trt": 0, "reg": 1, "bgk": 2}
WALLS = {"bb": 0, "bouzidi": 1}
STORAGES = {"f32": 0, "f16": 1, "bf16": 2}
LATERALS = {"periodic": 0, "free-slip": 3}  # slip.h: bit 0 y faces, bit 1 z faces


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp, u32, u16, f32, f64, sz, i32 = C.c_void_p, C.c_uint32, C.c_uint16, C.c_float, C.c_double, C.c_size_t, C.c_int
        sig = {
            "ow_f32_to_f16_rne": (u16, [f32]), "ow_f16_to_f32": (f32, [u16]),
            "ow_encode_f16": (u16, [f32, u32, u32]), "ow_encode_bf16": (u16, [f32, u32, u32]),
            "ow_f32_to_bf16_rne": (u16, [f32]), "ow_bf16_to_f32": (f32, [u16]),
            "ow_create": (vp, [u32, u32, u32, f32, f32, i32, i32, i32, i32, vp, sz, vp, sz, i32]),
            "ow_destroy": (None, [vp]), "ow_reset": (None, [vp, f32]),
            "ow_step": (None, [vp, f32, i32]), "ow_force": (None, [vp, vp]),
            "ow_populations": (None, [vp, vp]), "ow_populations_raw": (None, [vp, vp]),
            "ow_macros": (None, [vp, vp]), "ow_poke": (None, [vp, u32, u32, f32]),
            "ow_params": (None, [vp, vp]), "ow_set_lateral": (None, [vp, i32]),
            "oc_set_lateral": (None, [vp, i32, vp, sz, C.c_char_p, sz]),
            "oc_create": (vp, [u32, u32, u32, f64, i32, i32, vp, i32, vp, sz, vp, vp, i32, C.c_char_p, sz]),
            "oc_destroy": (None, [vp]), "oc_step": (None, [vp]),
            "oc_macroscopic": (None, [vp, u32, vp]), "oc_momentum_exchange": (None, [vp, vp]),
            "oc_populations": (C.POINTER(C.c_double), [vp]), "oc_cells": (sz, [vp]),
            "oc_equilibrium": (None, [vp, f64, vp]), "oc_moments": (None, [vp, vp]),
            "oc_collide": (None, [vp, vp, f64, f64, i32, i32, vp]),
            "oc_collide_wall": (i32, [vp, vp, f64, vp, vp, i32, f64, vp]),
            "oc_friction_velocity": (f64, [f64, f64]),
            "ov_voxelize": (i32, [vp, u32, vp, u32, i32, u32, u32, u32, i32, i32, vp, vp, vp, C.c_char_p, sz]),
            "ov_build_wall_links": (i32, [vp, vp, u32, vp, u32, i32, u32, u32, u32, i32, i32, vp, vp, vp]),
            "ov_free": (None, [vp]),
            "ov_nearest_link_hit": (i32, [vp, u32, u32, u32, u32, vp, vp, vp]),
            "ot_particles_update": (None, [vp, u32, vp, vp, u32, u32, u32, u32, f32, vp, vp]),
            "ot_hash": (u32, [u32]),
            "ot_plate_smoke": (None, [vp, u32, u32, u32, i32, vp, u32, u32, u32, u32, vp, vp, vp, u32]),
            "ot_streaks": (None, [vp, vp, u32, u32, u32, u32, i32, vp, f32, u32, u32, u32, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# ---------------------------------------------------------------- codecs
def encode_f16(value: float, i: int, n: int) -> int:
    return lib().ow_encode_f16(np.float32(value), i, n)


def encode_bf16(value: float, i: int, n: int) -> int:
    return lib().ow_encode_bf16(np.float32(value), i, n)


# ---------------------------------------------------------------- FP32 WGSL
class Wgsl32:
    """Binary32 restatement of the reference's WGSL kernels with A/B ping-pong."""

    def __init__(self, nx, ny, nz, tau0, u_in, geometry, boundary=None, les=False, op="trt",
                 walls="bb", storage="f32", threads=1, u_in_init=None, lateral="periodic"):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.cells = nx * ny * nz
        self.storage = storage
        g = np.ascontiguousarray(geometry, dtype=np.uint32)
        b = np.ascontiguousarray(boundary if boundary is not None else [], dtype=np.uint32)
        self._h = lib().ow_create(nx, ny, nz, np.float32(tau0), np.float32(u_in), int(les),
                                  OPERATORS[op], WALLS[walls], STORAGES[storage], _p(g), g.size,
                                  _p(b) if b.size else None, b.size, threads)
        if LATERALS[lateral]:
            lib().ow_set_lateral(self._h, LATERALS[lateral])
        if u_in_init is not None:
            self.reset(u_in_init)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ow_destroy(self._h)
            self._h = None

    def reset(self, u_in_init):
        lib().ow_reset(self._h, np.float32(u_in_init))

    def step(self, u_in, write_macro=False):
        lib().ow_step(self._h, np.float32(u_in), int(write_macro))

    def force(self):
        out = np.zeros(3, np.float64)
        lib().ow_force(self._h, _p(out))
        return out

    def populations(self):
        out = np.empty(19 * self.cells, np.float32)
        lib().ow_populations(self._h, _p(out))
        return out

    def populations_raw(self):
        out = np.empty(19 * self.cells, np.float32 if self.storage == "f32" else np.uint16)
        lib().ow_populations_raw(self._h, _p(out))
        return out

    def macros(self):
        out = np.empty(4 * self.cells, np.float32)
        lib().ow_macros(self._h, _p(out))
        return out

    def poke(self, i, n, value):
        lib().ow_poke(self._h, i, n, np.float32(value))

    def params(self):
        out = np.zeros(4, np.float32)
        lib().ow_params(self._h, _p(out))
        return out


# ---------------------------------------------------------------- FP64 CpuSolver
class Cpu64:
    """Binary64 restatement of the reference's CpuSolver."""

    def __init__(self, layout, tau0, operator="trt", les=False, body_force=(0.0, 0.0, 0.0),
                 walls="bb", flags=None, equilibrium_state=None, initial_state=None, threads=1,
                 lateral="periodic"):
        nx, ny, nz = layout
        self.layout = (nx, ny, nz)
        f = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint32)
        eq = None
        if equilibrium_state is not None:
            rho, u = equilibrium_state
            eq = np.array([rho, *u], np.float64)
        init = None if initial_state is None else np.ascontiguousarray(initial_state, np.float64).reshape(-1)
        bf = np.array(body_force, np.float64)
        err = C.create_string_buffer(256)
        self._keep = (f, eq, init, bf)
        self._h = lib().oc_create(nx, ny, nz, float(tau0), OPERATORS[operator], int(les), _p(bf),
                                  WALLS[walls], _p(f), 0 if f is None else f.size, _p(eq), _p(init),
                                  threads, err, 256)
        if not self._h:
            raise ValueError(err.value.decode())
        if LATERALS[lateral]:
            lib().oc_set_lateral(self._h, LATERALS[lateral], _p(f), 0 if f is None else f.size, err, 256)
            if err.value:
                raise ValueError(err.value.decode())
        self.cells = lib().oc_cells(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oc_destroy(self._h)
            self._h = None

    def step(self, n=1):
        for _ in range(n):
            lib().oc_step(self._h)

    @property
    def populations(self) -> np.ndarray:
        ptr = lib().oc_populations(self._h)
        return np.ctypeslib.as_array(ptr, shape=(19 * self.cells,))

    def macroscopic(self, cell):
        out = np.zeros(4, np.float64)
        lib().oc_macroscopic(self._h, cell, _p(out))
        return out[0], out[1:].copy()

    def macros(self):
        """(rho, ux, uy, uz) of every cell, computed like macroscopic()."""
        g = self.populations.reshape(19, self.cells)
        cx, cy, cz = LATTICE_C.T
        rho = 1.0 + np.zeros(self.cells)
        for i in range(19):
            rho = rho + g[i]
        m = [np.zeros(self.cells) for _ in range(3)]
        for i in range(19):
            m[0] = m[0] + cx[i] * g[i]
            m[1] = m[1] + cy[i] * g[i]
            m[2] = m[2] + cz[i] * g[i]
        return np.stack([rho, m[0] / rho, m[1] / rho, m[2] / rho], axis=1)

    def momentum_exchange(self):
        out = np.zeros(3, np.float64)
        lib().oc_momentum_exchange(self._h, _p(out))
        return out


LATTICE_C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                      [1, 1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, -1, -1],
                      [1, -1, 0], [-1, 1, 0], [1, 0, -1], [-1, 0, 1], [0, 1, -1], [0, -1, 1]])
LATTICE_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def equilibrium(rho, u):
    out = np.zeros(19)
    uu = np.array(u, np.float64)
    lib().oc_equilibrium(_p(out), float(rho), _p(uu))
    return out


def moments(g):
    g = np.ascontiguousarray(g, np.float64)
    out = np.zeros(4)
    lib().oc_moments(_p(g), _p(out))
    return out[0], out[1:].copy()


def collide(g, geq, rho, tau0, operator="trt", les=False, force_terms=None):
    g = np.ascontiguousarray(g, np.float64).copy()
    geq = np.ascontiguousarray(geq, np.float64)
    ft = np.zeros(19) if force_terms is None else np.ascontiguousarray(force_terms, np.float64)
    lib().oc_collide(_p(g), _p(geq), float(rho), float(tau0), OPERATORS[operator], int(les), _p(ft))
    return g


def collide_wall(g, geq, rho, u, wall_incoming, viscosity, force_terms=None):
    g = np.ascontiguousarray(g, np.float64).copy()
    geq = np.ascontiguousarray(geq, np.float64)
    uu = np.array(u, np.float64)
    wi = np.array(wall_incoming, np.int32)
    ft = np.zeros(19) if force_terms is None else np.ascontiguousarray(force_terms, np.float64)
    applied = lib().oc_collide_wall(_p(g), _p(geq), float(rho), _p(uu), _p(wi), wi.size,
                                    float(viscosity), _p(ft))
    return bool(applied), g


def friction_velocity(speed, viscosity):
    return lib().oc_friction_velocity(float(speed), float(viscosity))


# ---------------------------------------------------------------- geometry
class _Stats(C.Structure):
    _fields_ = [("solid_cells", C.c_uint32), ("frontal_cells", C.c_uint32),
                ("watertight", C.c_uint32), ("missed_links", C.c_uint32),
                ("blockage", C.c_double), ("geometry_len", C.c_size_t), ("nboundary", C.c_size_t)]


@dataclass
class OracleGrid:
    nx: int
    ny: int
    nz: int
    geometry: np.ndarray
    boundary_cells: np.ndarray
    solid_cells: int
    frontal_cells: int
    blockage: float
    watertight: bool
    missed_links: int


def _mesh(m):
    if m is None:
        return None, 0
    a = np.ascontiguousarray(m, np.float32).reshape(-1)
    if a.size % 9:
        raise ValueError("Mesh positions must match a non-negative triangle count.")
    return a, a.size // 9


def _take(ptr, n, dtype=np.uint32):
    arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint32)), shape=(max(n, 1),))[:n].copy()
    lib().ov_free(ptr)
    return arr.astype(dtype, copy=False)


def voxelize(body, supports, layout, floor, link_fractions=True) -> OracleGrid:
    nx, ny, nz = layout
    b, nb = _mesh(body)
    s, ns = _mesh(supports)
    if b is None:
        b = np.zeros(0, np.float32)
    gp, bp = C.c_void_p(), C.c_void_p()
    st = _Stats()
    err = C.create_string_buffer(256)
    rc = lib().ov_voxelize(_p(b), nb, _p(s), ns, int(s is not None), nx, ny, nz, int(floor),
                           int(link_fractions), C.byref(gp), C.byref(bp), C.byref(st), err, 256)
    if rc != 0:
        raise ValueError(err.value.decode())
    geometry = _take(gp, st.geometry_len)
    boundary = _take(bp, st.nboundary)
    return OracleGrid(nx, ny, nz, geometry, boundary, st.solid_cells, st.frontal_cells,
                      st.blockage, bool(st.watertight), st.missed_links)


def build_wall_links(flags, body, supports, layout, floor, measure=True):
    nx, ny, nz = layout
    f = np.ascontiguousarray(flags, np.uint32).copy()
    b, nb = _mesh(body)
    s, ns = _mesh(supports)
    gp, bp = C.c_void_p(), C.c_void_p()
    st = _Stats()
    lib().ov_build_wall_links(_p(f), _p(b), nb, _p(s), ns, int(s is not None), nx, ny, nz,
                              int(floor), int(measure), C.byref(gp), C.byref(bp), C.byref(st))
    return _take(gp, st.geometry_len), _take(bp, st.nboundary), st.missed_links


def nearest_link_hit(mesh, layout, origin, direction):
    m, nt = _mesh(mesh)
    o = np.array(origin, np.float64)
    d = np.array(direction, np.float64)
    t = C.c_double()
    hit = lib().ov_nearest_link_hit(_p(m), nt, *layout, _p(o), _p(d), C.byref(t))
    return t.value if hit else None


# ---------------------------------------------------------------- tracers
def particles_update(particles, macros, flags, layout, seed, steps, cross_section, fallback):
    p = np.ascontiguousarray(particles, np.float32).copy()
    m = np.ascontiguousarray(macros, np.float32)
    f = np.ascontiguousarray(flags, np.uint32)
    cs = np.array(cross_section, np.float32)
    fb = np.array(fallback, np.float32)
    lib().ot_particles_update(_p(p), p.size // 8, _p(m), _p(f), *layout, seed, np.float32(steps),
                              _p(cs), _p(fb))
    return p


def hash32(v):
    return lib().ot_hash(v & 0xFFFFFFFF)


def plate_smoke(smoke, threads, slots, release, releasing, rake, layout, plane, macros, flags, ports):
    s = np.ascontiguousarray(smoke, np.float32).copy()
    r = np.array(rake, np.float32)
    pt = np.ascontiguousarray(ports, np.float32).reshape(-1)
    lib().ot_plate_smoke(_p(s), threads, slots, release, int(releasing), _p(r), *layout, plane,
                         _p(np.ascontiguousarray(macros, np.float32)),
                         _p(np.ascontiguousarray(flags, np.uint32)), _p(pt), pt.size // 2)
    return s


def streaks(puffs, release_of, ry, rz, slots, release, releasing, rake, h, layout, macros, flags):
    p = np.ascontiguousarray(puffs, np.float32).copy()
    ro = np.ascontiguousarray(release_of, np.uint32).copy()
    r = np.array(rake, np.float32)
    lib().ot_streaks(_p(p), _p(ro), ry, rz, slots, release, int(releasing), _p(r), np.float32(h),
                     *layout, _p(np.ascontiguousarray(macros, np.float32)),
                     _p(np.ascontiguousarray(flags, np.uint32)))
    return p, ro
