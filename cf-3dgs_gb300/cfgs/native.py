"""ctypes binding of libcfgs.so (the C ABI declared in include/cfgs.h).

There is no fallback: if the library cannot be loaded, every caller gets an
ImportError/RuntimeError that says so.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

STATUS = {
    0: "CFGS_OK",
    1: "CFGS_ERR_INVALID_ARGUMENT",
    2: "CFGS_ERR_CAPACITY",
    3: "CFGS_ERR_LAUNCH",
    4: "CFGS_ERR_DEVICE_FLAG",
    5: "CFGS_ERR_TOO_LARGE",
}
FLAG_FRUSTUM_VIOLATION = 0x1
FLAG_CAPACITY_OVERFLOW = 0x2
FLAG_COPY_TIMEOUT = 0x4
FLAG_BARRIER_TIMEOUT = 0x8

_vp = C.c_void_p
_fp = C.c_void_p  # device float* passed as an address


class RenderSchedule(C.Structure):
    _fields_ = [("fwd_batch", C.c_int32), ("fwd_warps", C.c_int32), ("bwd_batch", C.c_int32), ("bin_launch", C.c_int32)]


class Settings(C.Structure):
    _fields_ = [
        ("image_height", C.c_int32),
        ("image_width", C.c_int32),
        ("tanfovx", C.c_float),
        ("tanfovy", C.c_float),
        ("bg", _fp),
        ("scale_modifier", C.c_float),
        ("viewmatrix", _fp),
        ("projmatrix", _fp),
        ("sh_degree", C.c_int32),
        ("campos", _fp),
        ("prefiltered", C.c_int32),
        ("debug", C.c_int32),
        ("schedule", RenderSchedule),
    ]


class Gaussians(C.Structure):
    _fields_ = [
        ("num_gaussians", C.c_int32),
        ("means3D", _fp),
        ("opacities", _fp),
        ("shs", _fp),
        ("sh_coeffs", C.c_int32),
        ("colors_precomp", _fp),
        ("scales", _fp),
        ("rotations", _fp),
        ("cov3D_precomp", _fp),
    ]


class Gradients(C.Structure):
    _fields_ = [
        ("dL_dmeans2D", _fp),
        ("dL_dcolors", _fp),
        ("dL_dopacity", _fp),
        ("dL_dmeans3D", _fp),
        ("dL_dcov3D", _fp),
        ("dL_dsh", _fp),
        ("dL_dscales", _fp),
        ("dL_drotations", _fp),
    ]


class Counts(C.Structure):
    _fields_ = [("num_rendered", C.c_uint32), ("flags", C.c_uint32)]


class BatchScene(C.Structure):
    _fields_ = [("image_width", C.c_int32), ("image_height", C.c_int32), ("tanfovx", C.c_float),
                ("tanfovy", C.c_float), ("viewmatrix", _fp), ("projmatrix", _fp), ("campos", _fp), ("bg", _fp),
                ("sh_degree", C.c_int32), ("sh_coeffs", C.c_int32), ("num_gaussians", C.c_int32)]


class BatchPlan(C.Structure):
    _fields_ = [("num_scenes", C.c_int32), ("num_blocks", C.c_int32), ("gauss_slots", C.c_int64),
                ("num_tiles", C.c_int32), ("pad_", C.c_int32), ("num_pixels", C.c_int64),
                ("desc_bytes", C.c_size_t), ("pose_state_bytes", C.c_size_t), ("geom_bytes", C.c_size_t),
                ("image_bytes", C.c_size_t)]


class BatchArgs(C.Structure):
    _fields_ = [("num_scenes", C.c_int32), ("num_blocks", C.c_int32), ("num_tiles", C.c_int32), ("pad_", C.c_int32),
                ("gauss_slots", C.c_int64), ("capacity", C.c_int64), ("descs", _vp), ("block_scene", _vp),
                ("tile_scene", _vp), ("means3D", _vp), ("opacities", _vp), ("shs", _vp), ("scales", _vp),
                ("rotations", _vp), ("target", _vp), ("color", _vp), ("radii", _vp), ("geom", _vp), ("image", _vp),
                ("binning", _vp), ("scratch", _vp), ("pose_partials", _vp), ("xi", _vp), ("adam_state", _vp),
                ("pose_states", _vp), ("lr", C.c_double), ("beta1", C.c_double), ("beta2", C.c_double),
                ("eps", C.c_double), ("schedule", RenderSchedule), ("sh_degree_bound", C.c_int32),
                ("pad2_", C.c_int32)]


EXPORTS = {
    # name: (restype, argtypes)
    "cfgs_geom_bytes": (C.c_size_t, [C.c_int32]),
    "cfgs_image_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
    "cfgs_binning_bytes": (C.c_size_t, [C.c_int64]),
    "cfgs_backward_scratch_bytes": (C.c_size_t, [C.c_int64]),
    "cfgs_geom_layout": (None, [C.c_int32, C.POINTER(C.c_size_t)]),
    "cfgs_image_layout": (None, [C.c_int32, C.c_int32, C.POINTER(C.c_size_t)]),
    "cfgs_binning_layout": (None, [C.c_int64, C.POINTER(C.c_size_t)]),
    "cfgs_preprocess_forward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, _vp]),
    "cfgs_read_counts": (C.c_int, [_vp, C.POINTER(Counts), _vp]),
    "cfgs_render_forward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, C.c_int64,
                                      _vp, _vp, _vp, _vp]),
    "cfgs_backward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, _vp, C.c_int64, _vp,
                                _vp, _vp, _vp, C.POINTER(Gradients), _vp]),
    "cfgs_bin_forward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, C.c_int64, _vp]),
    "cfgs_depth_order": (C.c_int, [C.c_int32, _vp, _vp]),
    "cfgs_bin_instances": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, C.c_int64, _vp]),
    "cfgs_composite_forward": (C.c_int, [C.POINTER(Settings), C.c_int32, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp,
                                         _vp]),
    "cfgs_render_backward": (C.c_int, [C.POINTER(Settings), C.c_int32, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp,
                                       _vp]),
    "cfgs_preprocess_backward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, C.c_int64, _vp,
                                           C.POINTER(Gradients), _vp]),
    "cfgs_mark_visible": (C.c_int, [C.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_pose_apply": (C.c_int, [C.c_int32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_pose_scratch_bytes": (C.c_size_t, [C.c_int32]),
    "cfgs_pose_grad": (C.c_int, [C.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_pose_adam": (C.c_int, [C.c_int32, _vp, _vp, _vp, C.c_double, C.c_double, C.c_double, C.c_double, _vp]),
    "cfgs_gaussian_adam": (C.c_int, [C.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_double, C.c_double,
                                     C.c_int64, _vp]),
    "cfgs_densify_stats": (C.c_int, [C.c_int64, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_densify_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "cfgs_densify_plan": (C.c_int, [C.c_int64, _vp, _vp, _vp, _vp, C.c_float, C.c_float, C.c_float, C.c_float,
                                    C.c_int32, _vp, _vp, _vp]),
    "cfgs_densify_write": (C.c_int, [C.c_int64, _vp, _vp, C.c_int32, _vp, _vp, C.c_int32, _vp, _vp, _vp, _vp,
                                     _vp]),
    "cfgs_depth_to_points": (C.c_int, [C.c_int32, C.c_int32, _vp, C.c_float, C.c_float, C.c_float, C.c_float, _vp,
                                       _vp]),
    "cfgs_pointcloud_workspace_bytes": (C.c_size_t, [C.c_int64]),
    "cfgs_knn3_mean_dist2": (C.c_int, [C.c_int64, _vp, _vp, _vp, _vp]),
    "cfgs_voxel_down_sample": (C.c_int, [C.c_int64, _vp, _vp, C.c_double, _vp, _vp, _vp, C.POINTER(C.c_int64),
                                         _vp]),
    "cfgs_ssim_scratch_bytes": (C.c_size_t, [C.c_int32, C.c_int32, C.c_int32]),
    "cfgs_ssim_forward": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_ssim_backward": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cfgs_render_schedule_check": (C.c_int, [C.POINTER(RenderSchedule), C.POINTER(RenderSchedule)]),
    "cfgs_diag_copy_timeout": (C.c_int, [C.c_uint32, _vp, _vp]),
    # include/cfgs_plain.h: the plain GPU path (published structure, comparison point)
    "cfgs_plain_work_bytes": (C.c_size_t, [C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
    "cfgs_plain_bin": (C.c_int, [C.POINTER(Settings), C.c_int32, _vp, _vp, C.c_int64, C.POINTER(C.c_int64), _vp]),
    "cfgs_plain_render_forward": (C.c_int, [C.POINTER(Settings), C.c_int32, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp,
                                            _vp]),
    "cfgs_plain_backward": (C.c_int, [C.POINTER(Settings), C.POINTER(Gaussians), _vp, _vp, _vp, _vp, C.c_int64, _vp,
                                      _vp, _vp, C.POINTER(Gradients), _vp]),
    "cfgs_l1_loss_scratch_bytes": (C.c_size_t, [C.c_int64]),
    "cfgs_l1_loss_forward": (C.c_int, [C.c_int64, _vp, _vp, C.c_int32, _vp, _vp, _vp, _vp]),
    "cfgs_l1_loss_backward": (C.c_int, [C.c_int64, _vp, _vp, C.c_int32, _vp, _vp, _vp]),
    "cfgs_batch_plan": (C.c_int, [C.c_int32, C.POINTER(BatchScene), _vp, C.POINTER(BatchPlan), _vp, _vp, _vp, _vp,
                                  _vp, _vp]),
    "cfgs_batch_init": (C.c_int, [C.POINTER(BatchArgs), _vp]),
    "cfgs_batch_iteration": (C.c_int, [C.POINTER(BatchArgs), _vp]),
}

_LIB = None


def lib_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Loads libcfgs.so (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if build_if_missing and (not path.exists() or os.environ.get("CFGS_NO_BUILD") != "1"):
        try:
            path = _build.build()
        except Exception as e:  # the toolkit is needed; say so instead of limping on
            if not path.exists():
                raise ImportError(f"libcfgs.so is missing and could not be built: {e}") from e
    if not path.exists():
        raise ImportError(f"libcfgs.so not found at {path}; run __graft_entry__.build()")
    lib = C.CDLL(str(path))
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int, what: str) -> None:
    if status != 0:
        raise RuntimeError(f"{what} failed: {STATUS.get(status, status)}")


GEOM_FIELDS = ["xy", "conic_op", "rgbd", "rect", "touched", "offset", "clamped", "block_sums", "depth_key",
               "depth_val", "rank_sums", "depth_counts", "depth_totals", "total"]
IMAGE_FIELDS = ["counts", "tile_count", "tile_range", "final_T", "n_contrib", "total"]
BINNING_FIELDS = ["key", "gid", "pidx", "sorted_gid", "sorted_pidx", "chunk_counts", "totals", "total"]


def geom_layout(n: int) -> dict:
    arr = (C.c_size_t * len(GEOM_FIELDS))()
    load().cfgs_geom_layout(int(n), arr)
    return dict(zip(GEOM_FIELDS, list(arr)))


def image_layout(w: int, h: int) -> dict:
    arr = (C.c_size_t * len(IMAGE_FIELDS))()
    load().cfgs_image_layout(int(w), int(h), arr)
    return dict(zip(IMAGE_FIELDS, list(arr)))


def binning_layout(cap: int) -> dict:
    arr = (C.c_size_t * len(BINNING_FIELDS))()
    load().cfgs_binning_layout(int(cap), arr)
    return dict(zip(BINNING_FIELDS, list(arr)))
