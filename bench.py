#!/usr/bin/env python3
"""Benchmark of the fused D3Q19 stream-collide on one GB300.

Workload: the bluff vehicle body scaled x4 into a 512 x 256 x 256 tunnel
(33,554,432 cells), regularized collision with Smagorinsky LES (C_s = 0.1) and the
Werner-Wengle wall model, floor on, u = 0.05, nu = 0.025 (Re 320 on the 160-cell
body), populations stored in FP16 (x 2^15, hash-dithered) -- the
headline -- with FP32 and BF16 storage measured in the same run.  A step is one
lattice update of every cell; the 2.5 GB (FP16) / 5.1 GB (FP32) population array
is far larger than the 129 MB L2, so no flush is needed between steps.

value   = MLUPS (million lattice-cell updates per second) of the FP16 kernel with
          state resident in HBM, timed with CUDA events on the solver's stream.
e2e     = the same metric through the public solver API the reference's headless
          runner uses (src/app/case-run.ts:154-169): host mesh -> GPU voxelizer ->
          create -> {step 8, encode force, read force} loop over --e2e-steps ->
          the velocity field read to the host (read velocity, gpu-solver.ts:338),
          wall clock, with the mesh upload, every force readback and the field
          readback inside the timed region; setup and readback times beside it.
roofline: the plain-cell kernels (the 32-bit cell-pair kernel, and on odd
          steps its seam-row variant), packed FP32 arithmetic, which update all
          but the wall-link and x-face cells: algorithmic bytes per cell update
          B = 2 * 19 * s + 1/8
          (s = 2 bytes; the 1/8 is the bit-packed special mask), achieved =
          their cells * B / their summed CUDA-event time per step, peak =
          measured HBM copy GB/s.  step_roofline repeats it for whole steps.
cpu_baseline: the binary64 restatement of the reference's CpuSolver (the
          reference's CPU path; the TypeScript original cannot run here), on all
          host cores, over a bounded number of full-domain steps.
accuracy: drag and field errors against that binary64 restatement: the sphere
          at Re 100 (96x48x48, FP32) and the 128x64x64 vehicle in each storage.
voxelizer: the reference's 200k-triangle voxelizer benchmark at 256x128x128;
tracers:  the 128x64x64 vehicle in frames of 8 steps with 3-D streaklines, the
          plate smoke and particles advanced after each frame; device times;
grid_check: the reference's three-tier grid check (GCI band) run one tier
          after another and with the three tiers side by side on one GPU;
batched_tunnels: 64 seeded tunnels of uneven size and Re, FP16 TRT, two
          concurrent persistent launches per step from captured graphs,
          autotuned shape;
          aggregate MLUPS and drag error against each tunnel alone in FP32.

--impl reference runs only that CPU path and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ = 512, 256, 256
SCALE = 4.0
U_IN = 0.05
NU = U_IN * 40 * SCALE / 320  # Re 320 on the body length (40 * SCALE cells)
TAU0 = 0.5 + 3 * NU


def set_size(nx):
    """The same case at nx x nx/2 x nx/2 with the body scaled by nx/128 (profiling runs)."""
    global NX, NY, NZ, SCALE, NU, TAU0
    NX, NY, NZ = nx, nx // 2, nx // 2
    SCALE = nx / 128
    NU = U_IN * 40 * SCALE / 320
    TAU0 = 0.5 + 3 * NU
METRIC = "D3Q19 MLUPS & % HBM roofline, FP16-store vs FP32, drag err vs FP64 at 1 GB300"
BYTES = {"f32": 2 * 19 * 4 + 0.125, "f16": 2 * 19 * 2 + 0.125, "bf16": 2 * 19 * 2 + 0.125}


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic():
    """Per-launch DRAM bytes of the FP16 step kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "stream_collide_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        text = self.file.read()
        os.unlink(self.file.name)
        return parse_clock_rows(text) or out


def parse_clock_rows(text):
    """Median SM clock, the highest maximum clock and the throttle reasons seen
    in `nvidia-smi --query-gpu=<ClockSampler.FIELDS> --format=csv,noheader,nounits`
    output; None when no row parses."""
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in text.strip().splitlines():
        r = line.split(",")
        try:
            sm.append(float(r[1]))
            mx.append(float(r[2]))
            for k, name in enumerate(names):
                if r[5 + k].strip().lower().startswith("active"):
                    reasons.add(name)
        except (ValueError, IndexError):
            continue
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def barrier(world):
    """All ranks meet here (replica runs); a no-op on one GPU."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(values, world):
    """Each value's maximum over the ranks: the slowest replica sets the job's time."""
    if world == 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_mlups(cells, steps, world, ms):
    """Whole-job MLUPS of `world` replicas that each updated `cells` cells
    `steps` times, the slowest taking `ms` milliseconds."""
    return cells * steps * world / (ms * 1e3)


def build_case():
    from pocketwind_gb300 import meshes
    return meshes.vehicle_case_mesh(NX, NY, SCALE)


def run_ours(args, rank, world):
    import numpy as np
    from pocketwind_gb300 import _lib
    from pocketwind_gb300.geometry import voxelize
    from pocketwind_gb300.solver import GpuSolver, SolverParams

    _lib.require_gpu()
    body = build_case()
    grid = voxelize(body, None, (NX, NY, NZ), True)
    cells = NX * NY * NZ
    results = {}
    for precision in args.only.split(","):
        solver = GpuSolver.create((NX, NY, NZ), grid, SolverParams(tau0=TAU0, u_in=U_IN, les=True, operator="reg",
                                                                   precision=precision))
        if isinstance(solver, Exception):
            raise solver
        solver.step(args.warmup)
        solver.time_steps(0)
        clocks = None
        if precision == "f16":
            sampler = ClockSampler()
            sampler.start()
        barrier(world)
        ms = solver.time_steps(args.steps)
        barrier(world)
        if precision == "f16":
            clocks = sampler.stop()
        kernel_ms = solver.profile_steps(min(args.steps, 200)) if precision == "f16" else None
        unstable = False
        solver.step(1, True)
        unstable = solver.guard_unstable()
        results[precision] = {"ms": ms, "clocks": clocks, "unstable": unstable, "kernel_ms": kernel_ms,
                              "profiled_steps": min(args.steps, 200)}
        solver.destroy()
    if args.no_e2e:
        return results, None, cells, grid
    # end-to-end through the public API (wall clock): mesh upload + voxelize + create,
    # then {step 8, encode force, read force} over the e2e steps, then the velocity
    # field read back to the host (read velocity: the macro buffer, 16 bytes a cell)
    import time as _t
    # the caller's result buffer for the velocity field, allocated and touched
    # once before the timed sequence, as a client keeps it (ordinary host
    # memory: on this Grace host, page-locked memory measured slower, 40 ms
    # against about 20 ms for the 537 MB field)
    field_host = np.zeros((NX * NY * NZ, 4), np.float32)
    barrier(world)
    t0 = _t.perf_counter()
    grid2 = voxelize(body, None, (NX, NY, NZ), True)
    solver = GpuSolver.create((NX, NY, NZ), grid2, SolverParams(tau0=TAU0, u_in=U_IN, les=True, operator="reg",
                                                                precision="f16"))
    t1 = _t.perf_counter()
    samples = max(1, args.e2e_steps // 8)
    for k in range(samples):
        solver.step(8, k == samples - 1)
        solver.encode_force()
        f = solver.read_force()
    t2 = _t.perf_counter()
    field = solver.macros(out=field_host)
    t3 = _t.perf_counter()
    barrier(world)
    finite = bool(np.isfinite(field).all())
    solver.destroy()
    e2e = {"total_s": t3 - t0, "setup_s": t1 - t0, "steps_s": t2 - t1, "readback_s": t3 - t2,
           "steps": samples * 8, "samples": samples, "mesh_bytes": body.positions.nbytes,
           "field_bytes": field.nbytes, "finite": finite}
    return results, e2e, cells, grid


def e2e_line(e2e, total_s, cells, world):
    """The e2e figure: MLUPS over the whole public-API sequence (mesh upload,
    voxelize, create, the sampled steps, the velocity field read back), with
    the setup and readback times beside it and the same sequence's MLUPS
    without the one-off setup."""
    if not e2e:
        return None
    steps = e2e["steps"]
    return {"value": round(job_mlups(cells, steps, world, total_s * 1e3), 2), "unit": "MLUPS",
            "h2d_bytes_per_step": round(e2e["mesh_bytes"] / steps, 2),
            "d2h_bytes_per_step": round((24 * e2e["samples"] + e2e["field_bytes"]) / steps, 2),
            "steps": steps, "setup_ms": round(1e3 * e2e["setup_s"], 2),
            "steps_ms": round(1e3 * e2e["steps_s"], 2), "read_velocity_ms": round(1e3 * e2e["readback_s"], 2),
            "mlups_after_setup": round(job_mlups(cells, steps, world, 1e3 * (e2e["steps_s"] + e2e["readback_s"])), 2),
            "sequence": "mesh upload + GPU voxelizer + create, then {step 8, encode force, read force} "
                        "(macros written on the last step), then the velocity field read into the "
                        "caller's host buffer",
            "field_finite": e2e["finite"]}


def accuracy_leg(steps, threads):
    """Drag and field errors against the binary64 CpuSolver restatement on the same
    voxel grids: the laminar sphere at Re 100 (96x48x48, FP32, TRT, free-slip
    lateral faces, 4,000 steps, drag averaged over steps 3,001-4,000) and the
    128x64x64 vehicle (REG + LES + wall model, floor) in each storage after
    `steps` steps."""
    import numpy as np
    from oracle import oracle as O
    from pocketwind_gb300 import cases, forces
    from pocketwind_gb300.solver import GpuSolver
    out = {}
    c = cases.sphere_case("free-slip")
    grid = c.grid()
    t0 = time.perf_counter()
    s = GpuSolver.create(c.layout, grid, c.params("f32"))
    fx, fy, fz = cases.mean_drag(cases.run_drag(s, c.steps), c.steps, c.average_steps)
    s.destroy()
    gpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    cpu = O.Cpu64(c.layout, c.tau0, flags=grid.flags, equilibrium_state=(1.0, (c.u_in, 0.0, 0.0)),
                  threads=threads, lateral=c.lateral)
    window = []
    for k in range(8, c.steps + 1, 8):
        cpu.step(8)
        if k > c.steps - c.average_steps:
            window.append(cpu.momentum_exchange()[0])
    cpu_s = time.perf_counter() - t0
    rfx = float(np.mean(window))
    out["sphere_re100"] = {"grid": "96x48x48", "storage": "f32", "operator": "trt", "lateral": "free-slip",
                           "steps": c.steps, "average_steps": c.average_steps, "fx": fx, "fx_fp64": rfx,
                           "drag_rel_err": abs(fx - rfx) / abs(rfx),
                           "cd": fx * forces.cd_per_lattice_force(grid.frontal_cells),
                           "frontal_cells": grid.frontal_cells,
                           # wall clock of the whole case, a force readback every 8 steps on both sides
                           "seconds": {"gpu": round(gpu_s, 3), "cpu_fp64": round(cpu_s, 3), "cpu_threads": threads}}
    # the same sphere with interpolated walls on measured link fractions (periodic
    # lateral faces), and halfway walls on that grid for comparison
    c = cases.sphere_case("periodic", walls="bouzidi")
    grid = c.grid()
    row = {"grid": "96x48x48", "storage": "f32", "operator": "trt", "lateral": "periodic",
           "steps": c.steps, "average_steps": c.average_steps, "frontal_cells": grid.frontal_cells,
           "missed_links": grid.missed_links}
    for walls in ("bouzidi", "bb"):
        p = c.params("f32")
        p.walls = walls
        s = GpuSolver.create(c.layout, grid, p)
        fx, fy, fz = cases.mean_drag(cases.run_drag(s, c.steps), c.steps, c.average_steps)
        s.destroy()
        row[walls] = {"fx": fx, "cd": fx * forces.cd_per_lattice_force(grid.frontal_cells)}
    cpu = O.Cpu64(c.layout, c.tau0, walls="bouzidi", flags=grid.geometry,
                  equilibrium_state=(1.0, (c.u_in, 0.0, 0.0)), threads=threads)
    window = []
    for k in range(8, c.steps + 1, 8):
        cpu.step(8)
        if k > c.steps - c.average_steps:
            window.append(cpu.momentum_exchange()[0])
    rfx = float(np.mean(window))
    row["bouzidi"]["fx_fp64"] = rfx
    row["bouzidi"]["drag_rel_err"] = abs(row["bouzidi"]["fx"] - rfx) / abs(rfx)
    out["sphere_re100_bouzidi"] = row
    v = cases.vehicle_case(128)
    grid = v.grid()
    cpu = O.Cpu64(v.layout, v.tau0, operator="reg", les=True, flags=grid.flags,
                  equilibrium_state=(1.0, (v.u_in, 0.0, 0.0)), threads=threads)
    cpu.step(steps)
    ref, fr = cpu.macros(), cpu.momentum_exchange()
    fluid = (grid.flags & 7) == 0
    per = {}
    for precision in ("f32", "f16", "bf16"):
        s = GpuSolver.create(v.layout, grid, v.params(precision))
        s.step(steps, True)
        m = s.macros().astype(np.float64)
        s.encode_force()
        f = s.read_force()
        s.destroy()
        per[precision] = {
            "u_l2_rel": float(np.linalg.norm((m[:, 1:] - ref[:, 1:])[fluid]) / np.linalg.norm(ref[:, 1:][fluid])),
            "rho_l2_rel": float(np.linalg.norm((m[:, 0] - ref[:, 0])[fluid]) / np.linalg.norm(ref[:, 0][fluid])),
            # the same difference against the density deviation rho - 1 (a far smaller norm)
            "rho_deviation_l2_rel": float(np.linalg.norm((m[:, 0] - ref[:, 0])[fluid]) /
                                          np.linalg.norm((ref[:, 0] - 1)[fluid])),
            "drag_rel_err": abs(f.fx - fr[0]) / abs(fr[0])}
    out["vehicle_128"] = {"grid": "128x64x64", "operator": "reg+les+wall model", "steps": steps, "storages": per}
    return out


def batch_leg(steps, sample_steps=200, count=64, peak=None):
    """64 independent tunnels (sizes, bodies and Re from splitmix64 seed 1), FP16
    storage, TRT, stepped as one batch: per step one persistent launch over all
    members' plain cells and one over their seam and edge cells beside it,
    replayed from captured 50-step graphs, launch shape from the autotuner.  Aggregate MLUPS over `steps` steps, then each member's drag over
    the last `sample_steps` steps against the same tunnel run alone in FP32."""
    import numpy as np
    from pocketwind_gb300 import cases, geometry, solver
    from pocketwind_gb300.batch import Batch
    tunnels = cases.batch_tunnels(count, 1)
    grids = [geometry.voxelize(t.body, None, t.layout, False) for t in tunnels]

    def make(i, precision):
        t = tunnels[i]
        return solver.GpuSolver.create(t.layout, grids[i], solver.SolverParams(
            tau0=t.tau0, u_in=0.05, operator="trt", precision=precision))

    members = [make(i, "f16") for i in range(count)]
    batch = Batch(members)
    tuning = batch.tune(8)
    batch.reset()
    ms = batch.time_steps(steps)
    cells = batch.cells

    def sampled(step, sols, every=8):
        acc = np.zeros(len(sols))
        for _ in range(sample_steps // every):
            step(every)
            for k, s in enumerate(sols):
                s.encode_force()
                acc[k] += s.read_force().fx
        return acc / (sample_steps // every)

    batch.reset()
    batch.step(steps - sample_steps)
    fx16 = sampled(batch.step, members)
    batch.destroy()
    for m in members:
        m.destroy()
    fx32 = np.zeros(count)
    for i in range(count):
        s = make(i, "f32")
        s.step(steps - sample_steps)
        fx32[i] = sampled(s.step, [s])[0]
        s.destroy()
    err = np.abs(fx16 - fx32) / np.abs(fx32)
    mlups = cells * steps / (ms * 1e3)
    out = {"domains": count, "cells": cells, "steps": steps, "storage": "f16", "operator": "trt",
           "ms_per_step": round(ms / steps, 4), "mlups": round(mlups, 1),
           "launches_per_step": 2, "graph_chunk_steps": 50,
           "tuning": {"blocks": tuning.blocks, "rows_per_item": tuning.rows_per_item,
                      "candidates": tuning.candidates},
           "drag_rel_err_vs_solo_f32": {"median": float(np.median(err)), "p90": float(np.percentile(err, 90)),
                                        "max": float(err.max()), "sample_steps": sample_steps}}
    if peak:
        out["hbm_frac"] = round(mlups * 1e6 * BYTES["f16"] / (peak * 1e9), 4)
    return out


def closure_leg(fine_steps, train_steps, threads, snapshots=8):
    """The learned closure: fine 256x128x128 vehicle runs (REG + LES + wall model,
    FP32) at Re 320, 640 and 1280 from seeded 1% velocity perturbations, each
    `fine_steps` long (20,480 = four flow-throughs by default), give 2x
    box-filtered samples from `snapshots` snapshots over the last two
    flow-throughs; the last snapshot of each Re is held out.  The network
    trains for `train_steps` Adam steps (batch 65,536, lr 1e-3); the 128x64x64
    grid at Re 640 then runs the same physical time (half the steps) with the
    closure and with plain Smagorinsky.  Drag coefficients (each grid's frontal
    area) are averaged over each run's last two flow-throughs, as the
    reference's validation cases average them (src/validation/cases.ts:101,240),
    and device times of the fine and coarse runs are compared.  A third coarse
    run without the plain cells' eddy viscosity gives the floor that no closure
    of this form can go below.  The three coarse runs are repeated with
    interpolated (Bouzidi) walls on the body (walls.wgsl:6-21), the wall
    treatment that responds to the coarse grid's resolution."""
    import numpy as np
    from pocketwind_gb300 import cases, forces, solver
    from pocketwind_gb300.closure import N_PARAMS, Closure
    net = Closure(1)
    out = {"fine_grid": "256x128x128", "coarse_grid": "128x64x64", "fine_steps": fine_steps,
           "train_steps": train_steps, "batch": 65536, "lr": 1e-3, "snapshots": snapshots}
    fine_cd = {}
    fine_ms = None
    held = []  # the last snapshot of each Re: held out of training
    fine_window = min(fine_steps, 2 * forces.flow_through_steps(256))
    for re in (320.0, 640.0, 1280.0):
        v = cases.vehicle_case(256)
        nu_f = 0.05 * v.length_cells / re
        grid = v.grid()
        s = solver.GpuSolver.create(v.layout, grid, solver.SolverParams(tau0=0.5 + 3 * nu_f, u_in=0.05, les=True,
                                                                         operator="reg"))
        cases.perturbed_start(s, grid, 0.05, 0.01, seed=int(re))
        lead = fine_steps - fine_window
        samples = cases.run_drag(s, lead) if lead else []
        per = fine_window // snapshots
        for k in range(snapshots):
            samples += cases.run_drag(s, per)
            s.step(1, True)  # a macro step for the snapshot
            start = net.dataset_size
            net.add_samples(s, nu_f / 2)
            if k == snapshots - 1:
                held.append((start, net.dataset_size))
        if re == 640.0:
            fx, _, _ = forces.averaged_forces(samples, s.step_count, fine_window)
            fine_cd[re] = fx * forces.cd_per_lattice_force(grid.frontal_cells)
            fine_ms = s.time_steps(200) / 200
        s.destroy()
    x, y = net.dataset()
    mask = np.zeros(len(y), bool)
    for a, b in held:
        mask[a:b] = True
    net.set_dataset(x[~mask], y[~mask])
    out["samples_train"], out["samples_held_out"] = int((~mask).sum()), int(mask.sum())
    first, last = net.train(train_steps, batch=65536, lr=1e-3)
    out["loss_first"], out["loss_last"] = first, last
    xh, yh = x[mask], y[mask]
    out["a_priori_mse_held_out"] = {"closure": float(np.mean((net.eval(xh) - yh) ** 2)),
                                    "smagorinsky": float(np.mean(yh * yh))}
    coarse = {}
    coarse_steps = fine_steps // 2
    coarse_window = min(coarse_steps, 2 * forces.flow_through_steps(128))
    # the floor of any closure that only scales the plain cells' eddy viscosity
    # by max(0, 1 + c): zero weights and output bias -1 remove it
    floor_net = Closure(1)
    w = np.zeros(N_PARAMS, np.float32)
    w[-1] = -1.0
    floor_net.params = w
    # the same three with interpolated (Bouzidi) walls on the coarse grid's body
    runs = [(label + suffix, attach, walls)
            for suffix, walls in (("", "bb"), ("_bouzidi", "bouzidi"))
            for label, attach in (("closure", net), ("smagorinsky", None), ("no_eddy_viscosity", floor_net))]
    for label, attach, walls in runs:
        c = cases.vehicle_case(128)
        c.walls = walls
        nu_c = 0.05 * c.length_cells / 640.0
        grid = c.grid()
        s = solver.GpuSolver.create(c.layout, grid, solver.SolverParams(tau0=0.5 + 3 * nu_c, u_in=0.05, les=True,
                                                                         operator="reg", walls=walls))
        if attach is not None:
            attach.attach(s)
        cases.perturbed_start(s, grid, 0.05, 0.01, seed=640)
        samples = cases.run_drag(s, coarse_steps)
        fx, _, _ = forces.averaged_forces(samples, coarse_steps, coarse_window)
        cd = fx * forces.cd_per_lattice_force(grid.frontal_cells)
        ms = s.time_steps(200) / 200
        coarse[label] = {"cd": cd, "ms_per_step": ms, "finite": bool(np.isfinite(s.macros()).all())}
        s.destroy()
    ref = fine_cd[640.0]
    for label in coarse:
        coarse[label]["cd_rel_err_vs_fine"] = abs(coarse[label]["cd"] - ref) / abs(ref)
        # the coarse grid covers the same physical time in half the steps
        coarse[label]["wall_time_ratio_fine_over_coarse"] = (2 * fine_ms) / coarse[label]["ms_per_step"]
    out["fine_cd_re640"] = ref
    out["average_window_flow_throughs"] = 2
    out["coarse_re640"] = coarse
    # device time of a closure step over a plain Smagorinsky step on the same grid
    out["closure_kernel"] = ("closure_pairs: the plain step's two-cell update with the network on two 128-cell "
                             "tcgen05 tiles per block; edge and floor kernels beside it")
    out["closure_over_plain_step"] = {
        walls: coarse["closure" + suffix]["ms_per_step"] / coarse["smagorinsky" + suffix]["ms_per_step"]
        for suffix, walls in (("", "halfway"), ("_bouzidi", "bouzidi"))}
    net.destroy()
    floor_net.destroy()
    return out


def grid_check_leg(run_flow_throughs):
    """The grid check (src/app/grid-check.ts): the sphere preset at a body
    length of 16 cells on tier S (128x64x64), 24 on M, 32 on L, Re 100 on the
    body length, REG + LES, FP16, `run_flow_throughs` flow-throughs per tier
    with the newest half averaged.  Wall time of the reference's order (one tier
    after another) against the three tiers stepped side by side on one GPU,
    and the band they give."""
    from pocketwind_gb300 import meshes, reporting

    def sphere_for(length, layout):
        return meshes.place_mesh(meshes.preset_mesh("sphere"), *layout, length, False)

    t0 = time.perf_counter()
    seq = reporting.run_grid_check(16, 128, reporting.gpu_tier_runner(sphere_for, re=100.0, floor=False),
                                   run_flow_throughs=run_flow_throughs)
    t1 = time.perf_counter()
    conc = reporting.gpu_grid_check(sphere_for, 16, 128, re=100.0, run_flow_throughs=run_flow_throughs, floor=False)
    t2 = time.perf_counter()
    band = conc.band
    return {"body": "sphere preset", "lengths_cells": [r.length_cells for r in conc.rows],
            "cd": [r.cd for r in conc.rows], "flow_throughs": run_flow_throughs,
            "band": ({"gci_pct": band.gci_pct, "extrapolated_cd": band.extrapolated_cd} if band.kind == "band"
                     else {"no_band": band.reason}),
            "rows_equal_one_at_a_time": conc.rows == seq.rows,
            "seconds_one_at_a_time": round(t1 - t0, 3), "seconds_side_by_side": round(t2 - t1, 3)}


def voxelizer_leg(iterations=5):
    """The reference's voxelizer benchmark (tests/unit/voxelize/voxelize.bench.ts):
    a 200,000-triangle sphere (the fixture's icosphere: 6 subdivisions plus
    39,360 extra splits, radius 18, centre (84.37, 64.23, 64.41)) voxelized at
    256 x 128 x 128 without a floor, with a 400 ms budget in the browser.  Wall
    clock of the whole call on the GPU (mesh upload, three parity-ray
    projections, wall links, q offsets, boundary list, statistics), best and
    median of `iterations` after one warm-up, beside the binary64 restatement
    on one host core; the two grids must be equal."""
    import numpy as np
    from oracle import oracle as O
    from pocketwind_gb300 import meshes
    from pocketwind_gb300.geometry import voxelize
    layout = (256, 128, 128)
    mesh = meshes.icosphere((84.37, 64.23, 64.41), 18, 6, 39360)
    times = []
    grid = None
    for _ in range(iterations + 1):
        t0 = time.perf_counter()
        grid = voxelize(mesh, None, layout, False)
        times.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    ref = O.voxelize(mesh.positions, None, layout, False, link_fractions=False)
    cpu_s = time.perf_counter() - t0
    timed = sorted(times[1:])
    return {"triangles": int(mesh.triangle_count), "grid": "256x128x128", "solid_cells": int(grid.solid_cells),
            "watertight": bool(grid.watertight), "ms_best": round(1e3 * timed[0], 2),
            "ms_median": round(1e3 * timed[len(timed) // 2], 2), "reference_budget_ms": 400,
            "cpu_binary64_one_core_ms": round(1e3 * cpu_s, 1),
            "equal_to_binary64_restatement": bool(np.array_equal(grid.geometry, ref.geometry))}


def tracer_leg(steps):
    """The tracers on the 128x64x64 vehicle (FP32, REG + LES, floor on), stepped
    in frames of 8 steps as the reference's frame loop does (src/app/run.ts:42,
    345), the macros written on each frame's last step.  After every frame: a
    16x16 rake of 3-D streaklines at x = 2 (512 puffs per nozzle), the plate
    smoke on the centre plane (36 rake threads and the 6 dye ports placed on
    the voxelized body, 8192 ring slots each; src/render/plate.ts:522-548) and
    65,536 particles seeded at x = 2 (src/render/particles.ts).  CUDA events
    on the domain's stream (torch.cuda.ExternalStream) time the frame's steps
    and each tracer kernel."""
    import numpy as np
    import torch
    from pocketwind_gb300 import cases, particle_layout as PAL, plate_layout as PL
    from pocketwind_gb300.solver import GpuSolver
    from pocketwind_gb300.tracers import Particles, PlateSmoke, Streaks

    case = cases.vehicle_case(128)
    grid = case.grid()
    layout = case.layout
    s = GpuSolver.create(layout, grid, case.params("f32"))
    if isinstance(s, Exception):
        raise s
    plane = layout[1] // 2
    pts = case.body.positions.reshape(-1, 3)
    # a desktop plate shows the whole z span that fitPlate gives it (plate-layout.ts:69)
    z_top = min(layout[2] - 2, max(1.9 * float(pts[:, 2].max()), 0.45 * layout[2]))
    low, high = PL.rake_span(z_top, layout[2])
    ports = PL.dye_ports(grid.flags, layout, plane, (low, high)).reshape(-1, 2)
    streaks = Streaks(s, 16, 16, 512, (2.0, 16.0, 48.0, 1.5, 30.0))
    plate = PlateSmoke(s, plane, PL.RAKE_THREADS, 8192, ports)
    seeds, region, fallback = PAL.particle_seeds(grid.flags, layout, pts.min(axis=0), pts.max(axis=0), 65536, 7)
    particles = Particles(s, seeds, 7, region, fallback)
    stream = torch.cuda.ExternalStream(s.buffers()[2])
    frames = max(1, steps // 8)
    total = np.zeros(4)
    rake = (float(PL.RAKE_X), low, high, 8.0)
    chunk = 50  # frames queued between host waits, so the host runs ahead of the device
    pending = []
    for frame in range(frames):
        release, releasing = frame // 2, frame % 2 == 0
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(stream)
        s.step(8, True)
        ev[1].record(stream)
        streaks.advance(8.0, release, releasing)
        ev[2].record(stream)
        plate.advance(release, releasing, rake)
        ev[3].record(stream)
        particles.update(8.0)
        ev[4].record(stream)
        if frame >= 8:  # the first frames warm the kernels up
            pending.append(ev)
        if len(pending) == chunk or frame == frames - 1:
            for e in pending:
                e[4].synchronize()
                total += [e[k].elapsed_time(e[k + 1]) for k in range(4)]
            pending = []
    timed = frames - min(frames, 8)
    puffs, _ = streaks.read()
    smoke = plate.read()
    recs = particles.read()
    unstable = s.guard_unstable()
    per = total / max(1, timed)
    out = {"case": "vehicle 128x64x64, FP32, REG + LES, floor", "frames": frames, "steps_per_frame": 8,
           "ms_per_frame": {"steps": per[0], "streaks": per[1], "plate_smoke": per[2], "particles": per[3]},
           "tracer_share_of_frame": float(per[1:].sum() / per.sum()) if per.sum() > 0 else None,
           "streaks": {"puffs": streaks.n, "live": int((puffs[:, 3] > 0).sum()),
                       "puff_advances_per_s": streaks.n / (per[1] * 1e-3) if per[1] > 0 else None},
           "plate_smoke": {"slots": int(smoke.shape[0]), "live": int((smoke[:, 3] > 0).sum()),
                           "slot_advances_per_s": smoke.shape[0] / (per[2] * 1e-3) if per[2] > 0 else None},
           "particles": {"count": int(recs.shape[0]), "finite": bool(np.isfinite(recs).all()),
                         "updates_per_s": recs.shape[0] / (per[3] * 1e-3) if per[3] > 0 else None},
           "unstable": unstable}
    for t in (particles, plate, streaks):
        t.destroy()
    s.destroy()
    return out


def cell_classes(flags):
    """Cells updated per step by the plain-cell kernels (plain fluid with
    1 <= x <= nx-2, and EQ cells without wall links) and by the edge kernel."""
    import numpy as np
    kind = flags & 7
    x = np.arange(flags.size, dtype=np.int64) % NX
    plain = ((flags == 0) & (x >= 1) & (x <= NX - 2)) | (flags == 4)
    fluid = (kind == 0) | (kind == 4)
    return int(plain.sum()), int((fluid & ~plain).sum())


def cpu_baseline(grid_flags, steps, threads):
    """Binary64 CpuSolver restatement on the host cores over `steps` full-domain steps."""
    from oracle import oracle as O
    s = O.Cpu64((NX, NY, NZ), TAU0, operator="reg", les=True, flags=grid_flags,
                equilibrium_state=(1.0, (U_IN, 0.0, 0.0)), threads=threads)
    t0 = time.perf_counter()
    s.step(steps)
    dt = time.perf_counter() - t0
    return NX * NY * NZ * steps / dt / 1e6, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--nx", type=int, default=512, help="profiling runs: the case at nx x nx/2 x nx/2")
    ap.add_argument("--only", default="f16,f32,bf16", help="profiling runs: storages to time (f16 first)")
    ap.add_argument("--no-e2e", action="store_true", help="profiling runs: skip the end-to-end leg")
    ap.add_argument("--e2e-steps", type=int, default=2000,
                    help="steps of the end-to-end leg (force read every 8, velocity field at the end)")
    ap.add_argument("--batch-steps", type=int, default=2000,
                    help="steps of the 64-tunnel batched leg (0 skips the leg)")
    ap.add_argument("--closure-steps", type=int, default=20480,
                    help="fine-grid steps of the learned-closure leg (0 skips the leg)")
    ap.add_argument("--closure-train-steps", type=int, default=20000, help="Adam steps of the closure leg")
    ap.add_argument("--voxelizer-iterations", type=int, default=5,
                    help="timed calls of the 200k-triangle voxelizer leg (0 skips the leg)")
    ap.add_argument("--tracer-steps", type=int, default=20000,
                    help="solver steps of the tracer leg, 8 per frame (0 skips the leg)")
    ap.add_argument("--grid-check-flow-throughs", type=float, default=4,
                    help="flow-throughs per tier of the grid-check leg (0 skips the leg)")
    ap.add_argument("--accuracy-steps", type=int, default=1000,
                    help="vehicle steps of the accuracy leg against FP64 (0 skips the leg)")
    args = ap.parse_args()
    if args.nx != 512:
        set_size(args.nx)
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        from pocketwind_gb300 import meshes
        from oracle import oracle as O
        body = build_case()
        g = O.voxelize(body.positions, None, (NX, NY, NZ), True, link_fractions=False)
        flags = g.geometry[: NX * NY * NZ]
        per = []
        cpu_steps = max(1, min(args.steps, args.cpu_steps))
        mlups, dt = cpu_baseline(flags, cpu_steps, threads)
        line = {"metric": METRIC, "value": round(mlups, 3), "unit": "MLUPS", "n_gpus": args.gpus,
                "steps": cpu_steps, "warmup": 0, "ms_per_step": round(1000 * dt / cpu_steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": f"vehicle body x{SCALE:g}, {NX}x{NY}x{NZ}, REG+LES+wall model, floor",
                           "cells": NX * NY * NZ},
                "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                                 "sample": f"{cpu_steps} full-domain steps of the binary64 CpuSolver restatement"},
                "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    results, e2e, cells, grid = run_ours(args, rank, world)
    ms, e2e_max = max_over_ranks([results["f16"]["ms"], e2e["total_s"] if e2e else 0.0], world)
    if rank != 0:
        return
    peak, peak_kind = read_peaks()
    mlups = job_mlups(cells, args.steps, world, ms)
    step_achieved = cells * BYTES["f16"] / (ms / args.steps / 1e3) / 1e9
    n_plain, n_edge = cell_classes(grid.flags)
    kms = results["f16"]["kernel_ms"]
    prof = results["f16"]["profiled_steps"]
    plain_s = (kms[0] + kms[1]) / prof / 1e3
    achieved = n_plain * BYTES["f16"] / plain_s / 1e9
    traffic = read_traffic()
    first = args.warmup + 1
    odd_steps = sum(1 for k in range(first, first + args.steps) if k % 2)
    launches = (args.steps - odd_steps) * (1 + (n_edge > 0)) + odd_steps * (2 + (n_edge > 0))
    line = {
        "metric": METRIC,
        "value": round(mlups, 2),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 arithmetic, f16 storage",
        "data": "synthetic (parametric bluff-body mesh)",
        "config": {"workload": f"vehicle body x{SCALE:g}, {NX}x{NY}x{NZ}, REG+LES+wall model, floor, FP16 storage",
                   "cells": cells, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (2.5 GB populations)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "kernel": "aa_step_pairs (+ aa_step_seam_pairs on odd steps): plain cells, two per thread",
                     "bytes_per_cell": BYTES["f16"], "cells_per_step": n_plain,
                     "ms_per_step": round(plain_s * 1e3, 4),
                     # the reference's own bench page also counts a 4-byte flag per cell
                     # (src/app/bench-page.ts:44-45): 80 bytes for 16-bit storage
                     "frac_reference_convention": round(achieved * 80.0 / BYTES["f16"] / peak, 4),
                     "traffic": traffic.get("bytes_per_step") if traffic else None,
                     "traffic_source": traffic.get("source") if traffic else None},
        "step_roofline": {"achieved": round(step_achieved, 1), "frac": round(step_achieved / peak, 4),
                          "kernel_shares": {"plain": round(kms[0] / sum(kms), 4), "seam_rows": round(kms[1] / sum(kms), 4),
                                            "edges": round(kms[2] / sum(kms), 4)},
                          "edge_cells": n_edge},
        "storage_sweep": {p: {"mlups": round(cells * args.steps / (r["ms"] * 1e3), 2),
                              "hbm_frac": round(cells * BYTES[p] / (r["ms"] / args.steps / 1e3) / 1e9 / peak, 4),
                              "stable": not r["unstable"]}
                          for p, r in results.items()},
        "e2e": e2e_line(e2e, e2e_max, cells, world),
        "gpu_launches": launches,
        "clocks": results["f16"]["clocks"],
    }
    line["roofline"]["step_frac"] = line["step_roofline"]["frac"]
    if "f32" in line["storage_sweep"]:
        line["storage_sweep"]["f16_over_f32"] = round(line["storage_sweep"]["f16"]["mlups"] /
                                                      line["storage_sweep"]["f32"]["mlups"], 3)
        line["roofline"]["f16_mlups"] = line["storage_sweep"]["f16"]["mlups"]
        line["roofline"]["f32_mlups"] = line["storage_sweep"]["f32"]["mlups"]
        line["roofline"]["f16_over_f32"] = line["storage_sweep"]["f16_over_f32"]
    if world == 1 and args.batch_steps > 0:
        line["batched_tunnels"] = batch_leg(args.batch_steps, peak=peak)
    if world == 1 and args.closure_steps > 0:
        line["learned_closure"] = closure_leg(args.closure_steps, args.closure_train_steps, os.cpu_count() or 1)
    if world == 1 and args.voxelizer_iterations > 0:
        line["voxelizer"] = voxelizer_leg(args.voxelizer_iterations)
    if world == 1 and args.tracer_steps > 0:
        line["tracers"] = tracer_leg(args.tracer_steps)
    if world == 1 and args.grid_check_flow_throughs > 0:
        line["grid_check"] = grid_check_leg(args.grid_check_flow_throughs)
    if world == 1 and args.accuracy_steps > 0:
        line["accuracy"] = accuracy_leg(args.accuracy_steps, os.cpu_count() or 1)
    if world == 1 and args.cpu_steps > 0:
        flags = grid.flags.copy()
        cmlups, cdt = cpu_baseline(flags, args.cpu_steps, os.cpu_count() or 1)
        one, one_dt = cpu_baseline(flags, 1, 1)  # the reference's CPU path is single-threaded JavaScript
        line["cpu_baseline"] = {"value": round(cmlups, 3), "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{args.cpu_steps} full-domain steps of the binary64 CpuSolver "
                                          f"restatement ({cdt:.1f} s)",
                                "single_thread": {"value": round(one, 3), "cores": 1,
                                                  "sample": f"1 full-domain step ({one_dt:.1f} s)"}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
