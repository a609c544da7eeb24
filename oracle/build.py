"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the C restatements in this directory into ``oracle/_build/libpw_oracle.so``
with gcc.  ``-ffp-contract=off`` keeps every binary32/binary64 product and sum a
separate IEEE operation (gcc contracts a*b+c into fma by default on aarch64), so
the oracle evaluates the reference's expressions in the reference's order.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = ["lbm_f32.c", "lbm_f64.c", "geometry.c", "tracers.c"]
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libpw_oracle.so"
CFLAGS = [
    "-O2", "-std=gnu11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
    "-fno-strict-aliasing", "-Wall", "-Wno-unused-function",
]


def _stale() -> bool:
    if not LIB.exists():
        return True
    built = LIB.stat().st_mtime
    deps = [HERE / s for s in SOURCES] + [HERE / "pw_oracle.h", Path(__file__)]
    return any(d.stat().st_mtime > built for d in deps)


def build(force: bool = False) -> Path:
    """Compile the oracle shared library if any source is newer than it."""
    if not force and not _stale():
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    tmp = OUT_DIR / f"libpw_oracle.{os.getpid()}.so"
    cmd = ["gcc", *CFLAGS, "-shared", "-o", str(tmp)] + [str(HERE / s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
