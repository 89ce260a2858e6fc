"""Builds libcfgs.so, the sm_103a rasteriser library, in-tree.

Each CUDA translation unit is compiled by nvcc in parallel for exactly one target
(``-gencode arch=compute_103a,code=sm_103a``) and linked into one shared library
against the shared CUDA runtime, so that the library and PyTorch use the same runtime
instance (streams created by torch are valid in the library).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent            # cf-3dgs_gb300/cfgs
SRC_DIR = PKG_DIR.parent / "csrc"                    # cf-3dgs_gb300/csrc
INCLUDE_DIR = PKG_DIR.parent.parent / "include"      # repo include/
BUILD_DIR = PKG_DIR / "_build"
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libcfgs.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                "--expt-relaxed-constexpr", f"-I{INCLUDE_DIR}"]
# Translation units whose float results the CPU oracle reproduces bit for bit are
# compiled without FMA contraction; their fused operations are explicit fmaf() calls.
NO_CONTRACT = {"preprocess.cu", "render_fwd.cu"}
SOURCES = ["preprocess.cu", "binning.cu", "render_fwd.cu", "render_bwd.cu", "preprocess_bwd.cu", "pose.cu", "batch.cu", "ssim.cu", "pointcloud.cu", "densify.cu", "loss.cu"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcfgs.so")
    return cand


def _cuda_lib_dir(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent / "lib64"


def _compile(nvcc: str, src: str, extra: list[str]) -> Path:
    obj = BUILD_DIR / (Path(src).stem + ".o")
    flags = list(COMMON_FLAGS) + list(ARCH_FLAGS) + list(extra)
    if src in NO_CONTRACT:
        flags.append("-fmad=false")
    cmd = [nvcc, "-c", str(SRC_DIR / src), "-o", str(obj)] + flags
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = [SRC_DIR / s for s in SOURCES] + list(SRC_DIR.glob("*.cuh")) + list(INCLUDE_DIR.glob("*.h"))
    deps.append(Path(__file__))
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles (if stale) and returns the path of libcfgs.so."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    extra = list(extra_flags or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    libdir = _cuda_lib_dir(nvcc)
    cmd = [nvcc, "-shared", "-cudart", "shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH_FLAGS + [
        f"-L{libdir}", "-Xlinker", f"-rpath={libdir}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
