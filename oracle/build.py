"""Build recipe of the CPU oracle library (test infrastructure only).

gcc, C11, no FMA contraction and no fast-math: the oracle's float results depend on
every operation being rounded exactly as written. OpenMP parallelises the per-Gaussian
and per-tile loops (the results do not depend on the thread count).
"""
from __future__ import annotations

import hashlib
import os
import platform
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


STAMP = OUT_DIR / "libcfgs_oracle.stamp"


def _fingerprint(cc: str | None) -> str:
    """Hash of the sources, this recipe, the flags, the compiler and the host
    architecture; the library is rebuilt whenever its stamp differs."""
    h = hashlib.sha256()
    for p in SRCS + [Path(__file__)]:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(repr(FLAGS).encode())
    h.update(platform.machine().encode())
    h.update((cc or "").encode())
    return h.hexdigest()


def build(force: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    fp = _fingerprint(cc)
    if not force and LIB.exists() and STAMP.exists() and STAMP.read_text().strip() == fp:
        return LIB
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc] + FLAGS + [str(p) for p in SRCS] + ["-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    STAMP.write_text(fp + "\n")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
