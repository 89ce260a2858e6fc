"""Build recipe of the CPU oracle library (test infrastructure only).

gcc, C11, no FMA contraction and no fast-math: the oracle's float results depend on
every operation being rounded exactly as written. OpenMP parallelises the per-Gaussian
and per-tile loops (the results do not depend on the thread count).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cfgs_oracle.c"
SRCS = [SRC, HERE / "pointcloud_oracle.c"]
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libcfgs_oracle.so"
FLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fopenmp", "-Wall",
         "-Wno-unknown-pragmas"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max([p.stat().st_mtime for p in SRCS] + [Path(__file__).stat().st_mtime]):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc] + FLAGS + [str(p) for p in SRCS] + ["-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
