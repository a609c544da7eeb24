"""Build libpocketwind_gb300.so in-tree for sm_103a (GB300).

Each translation unit compiles in parallel with nvcc; the product links into
``pocketwind_gb300/_build/libpocketwind_gb300.so`` (git-ignored).  Units whose
binary32/binary64 rounding must follow the reference's expression order (the
strict stream-collide build, the voxelizer and the tracers) compile with
``-fmad=false``; the fast stream-collide build keeps fused multiply-add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libpocketwind_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{INCLUDE}", "--expt-relaxed-constexpr"]
UNITS = {
    "pw_kernels_fast.cu": [],
    "pw_kernels_strict.cu": ["-fmad=false"],
    "pw_geometry.cu": ["-fmad=false"],
    "pw_tracers.cu": ["-fmad=false"],
    "pw_domain.cu": [],
    "pw_noalloc.cu": [],
    "pw_batch.cu": [],
    "pw_closure.cu": [],
}
HEADERS = ["pw_common.cuh", "pw_lbm.cuh", "pw_lbm_tile.cuh", "pw_launch.h", "pw_internal.h", "pw_closure.cuh"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libpocketwind_gb300")
    return exe


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / u for u in UNITS] + [CSRC / h for h in HEADERS] + [INCLUDE / "pocketwind.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_unit(name: str) -> Path:
        obj = OUT / (name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], "-c", str(CSRC / name), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = OUT / f"libpocketwind_gb300.{os.getpid()}.so"
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
