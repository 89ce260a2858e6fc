"""Local-Gaussian initialisation of a CF-3DGS frame on the GPU (the steps before each
pose solve): depth -> points (kornia depth_to_3d, trainer/trainer.py:491), voxel
down-sampling (Open3D voxel_down_sample, trainer/trainer.py:507), initial scales from
the three nearest neighbours (simple-knn distCUDA2, scene/gaussian_model_cf.py:194) and
the initial Gaussian parameters of create_from_pcd (scene/gaussian_model_cf.py:175-210).
Every step calls libcfgs.so; CUDA tensors in, CUDA tensors out."""
from __future__ import annotations

import math

import torch

from . import native
from .raster import _ptr, stream_handle

C0 = 0.28209479177387814  # utils/sh_utils.py: SH band-0 constant


def _cuda_f32(t: torch.Tensor, what: str) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError(f"{what}: expected a CUDA tensor")
    return t.float().contiguous()


def depth_to_points(depth: torch.Tensor, K) -> torch.Tensor:
    """[H,W] depth and 3x3 intrinsics -> [H*W,3] camera-space points, row-major pixels
    (kornia depth_to_3d with normalize_points=False, permuted to [H*W,3])."""
    d = _cuda_f32(depth, "depth_to_points")
    H, W = (int(x) for x in d.shape[-2:])
    Km = torch.as_tensor(K, dtype=torch.float64).reshape(3, 3)
    fx, fy, cx, cy = float(Km[0, 0]), float(Km[1, 1]), float(Km[0, 2]), float(Km[1, 2])
    out = torch.empty((H * W, 3), dtype=torch.float32, device=d.device)
    native.check(native.load().cfgs_depth_to_points(H, W, _ptr(d), fx, fy, cx, cy, _ptr(out),
                                                    stream_handle(d.device)), "cfgs_depth_to_points")
    return out


def _workspace(n: int, device) -> torch.Tensor:
    return torch.empty(int(native.load().cfgs_pointcloud_workspace_bytes(n)), dtype=torch.uint8, device=device)


def voxel_down_sample(points: torch.Tensor, colors: torch.Tensor | None = None, voxel_size: float = 0.01):
    """Averages the points (and colours) of every occupied voxel of edge voxel_size
    (Open3D voxel_down_sample). Voxels come out in increasing voxel index order."""
    p = _cuda_f32(points, "voxel_down_sample").reshape(-1, 3)
    c = None if colors is None else _cuda_f32(colors, "voxel_down_sample").reshape(-1, 3)
    n = int(p.shape[0])
    op = torch.empty_like(p)
    oc = None if c is None else torch.empty_like(c)
    m = native.C.c_int64(0)
    ws = _workspace(n, p.device)
    native.check(native.load().cfgs_voxel_down_sample(n, _ptr(p), _ptr(c), float(voxel_size), _ptr(ws), _ptr(op),
                                                      _ptr(oc), native.C.byref(m), stream_handle(p.device)),
                 "cfgs_voxel_down_sample")
    k = int(m.value)
    return op[:k], (None if oc is None else oc[:k])


def dist_cuda2(points: torch.Tensor) -> torch.Tensor:
    """Per point the mean squared distance to its three nearest other points
    (simple-knn distCUDA2)."""
    p = _cuda_f32(points, "dist_cuda2").reshape(-1, 3)
    n = int(p.shape[0])
    out = torch.empty(n, dtype=torch.float32, device=p.device)
    ws = _workspace(n, p.device)
    native.check(native.load().cfgs_knn3_mean_dist2(n, _ptr(p), _ptr(ws), _ptr(out), stream_handle(p.device)),
                 "cfgs_knn3_mean_dist2")
    return out


def gaussians_from_points(points: torch.Tensor, colors: torch.Tensor, sh_degree: int = 3,
                          view_dependent: bool = False) -> dict:
    """create_from_pcd (scene/gaussian_model_cf.py:175-210): colours as the DC term
    (RGB2SH when view-dependent), scales log(sqrt(max(dist2, 1e-7))) on all three axes,
    identity rotations, opacity logit of 0.1."""
    p = _cuda_f32(points, "gaussians_from_points").reshape(-1, 3)
    col = _cuda_f32(colors, "gaussians_from_points").reshape(-1, 3)
    n = p.shape[0]
    dc = (col - 0.5) / C0 if view_dependent else col
    features = torch.zeros((n, 3, (sh_degree + 1) ** 2), dtype=torch.float32, device=p.device)
    features[:, :3, 0] = dc
    dist2 = torch.clamp_min(dist_cuda2(p), 0.0000001)
    scales = torch.log(torch.sqrt(dist2))[..., None].repeat(1, 3)
    rots = torch.zeros((n, 4), dtype=torch.float32, device=p.device)
    rots[:, 0] = 1
    opacities = torch.full((n, 1), math.log(0.1 / 0.9), dtype=torch.float32, device=p.device)
    return {"xyz": p.clone(), "features_dc": features[:, :, 0:1].transpose(1, 2).contiguous(),
            "features_rest": features[:, :, 1:].transpose(1, 2).contiguous(), "scaling": scales,
            "rotation": rots, "opacity": opacities}
