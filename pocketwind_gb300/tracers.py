"""Tracers advected by a solver's macro field (library kernels, no host fallback).

* ``Particles``  -- src/render/particles.ts + particles_update.wgsl: 3-D trilinear
  velocity, Euler step capped at one cell, hash respawn at x = 2 (8 floats per
  record: pos.xyz, age, prev.xyz, generation).
* ``PlateSmoke`` -- src/render/plate.ts:522-548 + plate_smoke.wgsl: rake and dye-port
  threads on one y plane, ring of slots, RK2 with slide and settle; records
  (x, z, release index, density).
* ``Streaks``    -- 3-D streaklines: a ry x rz rake, ring of ``slots`` puffs per
  nozzle, trilinear RK2 with the plate's sub-step, cap, slide and settle rules;
  records (x, y, z, density) plus the release index of each slot.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .solver import GpuSolver

RAKE_THREADS = 36      # plate-layout.ts:5
PORTS = 6              # plate-layout.ts:15
RING_SLOTS = 8192      # plate-layout.ts:23
RELEASE_EVERY_FRAMES = 2


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


class Particles:
    def __init__(self, solver: GpuSolver, records: np.ndarray, seed: int, cross_section, fallback):
        self._ptr = None
        rec = np.ascontiguousarray(records, np.float32).reshape(-1)
        if rec.size % 8:
            raise _lib.RangeError("Particle records hold 8 floats.")
        self.count = rec.size // 8
        cs = np.array(cross_section, np.float32)
        fb = np.array(fallback, np.float32)
        out = C.c_void_p()
        self.solver = solver
        _lib.check(_lib.load().pw_particles_create(solver._live(), _vp(rec), self.count, int(seed), _vp(cs), _vp(fb),
                                                   C.byref(out)), "particles")
        self._ptr = out.value

    def update(self, steps: float) -> None:
        self.solver._live()
        _lib.check(_lib.load().pw_particles_update(self._ptr, float(steps)), "particles update")

    def write(self, records: np.ndarray) -> None:
        rec = np.ascontiguousarray(records, np.float32).reshape(-1)
        _lib.check(_lib.load().pw_particles_write(self._ptr, _vp(rec)), "particles write")

    def read(self) -> np.ndarray:
        out = np.empty((self.count, 8), np.float32)
        _lib.check(_lib.load().pw_particles_read(self._ptr, _vp(out)), "particles read")
        return out

    def destroy(self):
        if self._ptr:
            _lib.load().pw_particles_destroy(self._ptr)
            self._ptr = None

    __del__ = destroy


class PlateSmoke:
    def __init__(self, solver: GpuSolver, plane: int, rake_threads: int = RAKE_THREADS,
                 slots: int = RING_SLOTS, ports=None):
        self._ptr = None
        pts = np.zeros(0, np.float32) if ports is None else np.ascontiguousarray(ports, np.float32).reshape(-1)
        self.threads = rake_threads + pts.size // 2
        self.slots = slots
        out = C.c_void_p()
        self.solver = solver  # the plate samples the solver's buffers: keep it alive
        _lib.check(_lib.load().pw_plate_create(solver._live(), int(plane), rake_threads, slots,
                                               _vp(pts) if pts.size else None, pts.size // 2, C.byref(out)), "plate")
        self._ptr = out.value

    def advance(self, release: int, releasing: bool, rake) -> None:
        self.solver._live()
        r = np.array(rake, np.float32)
        _lib.check(_lib.load().pw_plate_advance(self._ptr, int(release), int(bool(releasing)), _vp(r)), "plate advance")

    def read(self) -> np.ndarray:
        out = np.empty((self.threads * self.slots, 4), np.float32)
        _lib.check(_lib.load().pw_plate_read(self._ptr, _vp(out)), "plate read")
        return out

    def destroy(self):
        if self._ptr:
            _lib.load().pw_plate_destroy(self._ptr)
            self._ptr = None

    __del__ = destroy


class Streaks:
    def __init__(self, solver: GpuSolver, ry: int, rz: int, slots: int, rake):
        self._ptr = None
        r = np.array(rake, np.float32)
        out = C.c_void_p()
        self.n = ry * rz * slots
        self.solver = solver  # the streaks sample the solver's buffers: keep it alive
        _lib.check(_lib.load().pw_streaks_create(solver._live(), ry, rz, slots, _vp(r), C.byref(out)), "streaks")
        self._ptr = out.value

    def advance(self, h_steps: float, release: int, releasing: bool) -> None:
        self.solver._live()
        _lib.check(_lib.load().pw_streaks_advance(self._ptr, float(h_steps), int(release), int(bool(releasing))),
                   "streaks advance")

    def read(self):
        puffs = np.empty((self.n, 4), np.float32)
        rel = np.empty(self.n, np.uint32)
        _lib.check(_lib.load().pw_streaks_read(self._ptr, _vp(puffs), _vp(rel)), "streaks read")
        return puffs, rel

    def destroy(self):
        if self._ptr:
            _lib.load().pw_streaks_destroy(self._ptr)
            self._ptr = None

    __del__ = destroy
