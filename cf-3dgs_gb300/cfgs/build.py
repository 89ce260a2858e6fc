"""Builds libcfgs.so, the sm_103a rasteriser library, in-tree.

Each CUDA translation unit is compiled by nvcc in parallel for exactly one target
(``-gencode arch=compute_103a,code=sm_103a``) and linked into one shared library
against the shared CUDA runtime, so that the library and PyTorch use the same runtime
instance (streams created by torch are valid in the library).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
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
NO_CONTRACT = {"preprocess.cu", "render_fwd.cu", "plain_raster.cu"}
SOURCES = ["preprocess.cu", "binning.cu", "render_fwd.cu", "render_bwd.cu", "preprocess_bwd.cu", "pose.cu", "batch.cu", "ssim.cu", "pointcloud.cu", "densify.cu", "loss.cu", "plain_raster.cu"]


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


STAMP_PATH = LIB_DIR / "libcfgs.stamp"


def _fingerprint(nvcc: str | None, extra: list[str]) -> str:
    """Hash of everything the library is built from: every source and header, this
    recipe, the flags, the compiler's version line and the host architecture. A library
    whose stamp differs (edited sources, other flags, a copy built on another machine) is
    rebuilt, whatever the files' modification times say."""
    h = hashlib.sha256()
    deps = [SRC_DIR / s for s in SOURCES] + sorted(SRC_DIR.glob("*.cuh")) + sorted(INCLUDE_DIR.glob("*.h"))
    deps.append(Path(__file__))
    for p in deps:
        h.update(p.name.encode())
        h.update(p.read_bytes() if p.exists() else b"<missing>")
    h.update(repr((COMMON_FLAGS, ARCH_FLAGS, sorted(NO_CONTRACT), extra)).encode())
    h.update(platform.machine().encode())
    if nvcc:
        try:
            out = subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout
            h.update(out.strip().splitlines()[-1].encode() if out.strip() else b"")
        except OSError:
            pass
    return h.hexdigest()


def _stale(fingerprint: str) -> bool:
    if not LIB_PATH.exists() or not STAMP_PATH.exists():
        return True
    return STAMP_PATH.read_text().strip() != fingerprint


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compiles (when the library's stamp does not match its sources, flags and
    toolchain) and returns the path of libcfgs.so."""
    extra = list(extra_flags or [])
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    fp = _fingerprint(nvcc if Path(nvcc).exists() else None, extra)
    if not force and not _stale(fp):
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
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
    STAMP_PATH.write_text(fp + "\n")
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
