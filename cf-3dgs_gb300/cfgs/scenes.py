"""Cameras and seeded synthetic scenes for the rasteriser and pose-solve workloads.

Camera matrices follow the intrinsics branch of the reference Camera
(scene/cameras.py:57-74, `is_co3d`): world_view_transform = getWorld2View3(R, T)^T
(utils/graphics_utils.py:69-82), an OpenGL-style projection built from (fx, fy, cx, cy)
with znear 0.01 / zfar 100 (scene/cameras.py:51-52,61-67), full = view @ proj, and the
camera centre = inverse(view)[3, :3].

The scenes stand in for the datasets the reference trains on (Tanks&Temples, CO3D),
which are not available: their shapes and value distributions are the ones the
workload definitions name, drawn from numpy's seeded generator.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

SH_C0 = 0.28209479177387814


@dataclass
class Camera:
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    viewmatrix: torch.Tensor      # [4,4] float32, world_view_transform
    projmatrix: torch.Tensor      # [4,4] float32, full_proj_transform
    campos: torch.Tensor          # [3]
    tanfovx: float
    tanfovy: float

    def to(self, device) -> "Camera":
        return Camera(self.width, self.height, self.fx, self.fy, self.cx, self.cy, self.viewmatrix.to(device),
                      self.projmatrix.to(device), self.campos.to(device), self.tanfovx, self.tanfovy)


def make_camera(width: int, height: int, fx: float, fy: float, cx: float | None = None, cy: float | None = None,
                R: np.ndarray | None = None, T: np.ndarray | None = None, znear: float = 0.01,
                zfar: float = 100.0) -> Camera:
    cx = width / 2.0 if cx is None else cx
    cy = height / 2.0 if cy is None else cy
    R = np.eye(3) if R is None else np.asarray(R, dtype=np.float64)
    T = np.zeros(3) if T is None else np.asarray(T, dtype=np.float64)
    Rt = np.zeros((4, 4))
    Rt[:3, :3] = R
    Rt[:3, 3] = T
    Rt[3, 3] = 1.0
    c2w = np.linalg.inv(Rt)
    w2c = np.linalg.inv(c2w).astype(np.float32)
    view = torch.tensor(w2c).transpose(0, 1).contiguous()
    w, h = float(width), float(height)
    proj = torch.tensor([[2 * fx / w, 0.0, -(w - 2 * cx) / w, 0.0],
                         [0.0, 2 * fy / h, -(h - 2 * cy) / h, 0.0],
                         [0.0, 0.0, zfar / (zfar - znear), -(zfar * znear) / (zfar - znear)],
                         [0.0, 0.0, 1.0, 0.0]], dtype=torch.float32).transpose(0, 1)
    full = (view.unsqueeze(0).bmm(proj.unsqueeze(0))).squeeze(0).contiguous()
    campos = view.inverse()[3, :3].contiguous()
    fovx = 2 * math.atan(width / (2 * fx))
    fovy = 2 * math.atan(height / (2 * fy))
    return Camera(width, height, fx, fy, cx, cy, view, full, campos, math.tan(fovx * 0.5), math.tan(fovy * 0.5))


@dataclass
class Scene:
    """Activated Gaussian parameters, as CF3DGS_Render.render passes them to the
    rasteriser (scene/gaussian_model_cf.py:828-868)."""
    means3D: torch.Tensor          # [N,3]
    opacities: torch.Tensor        # [N,1] sigmoid-activated
    shs: torch.Tensor              # [N,M,3]
    scales: torch.Tensor           # [N,3] exp-activated
    rotations: torch.Tensor        # [N,4] unit quaternion (r,x,y,z)
    sh_degree: int
    camera: Camera
    target: torch.Tensor | None = None   # [3,H,W]
    bg: torch.Tensor = field(default_factory=lambda: torch.zeros(3))
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.means3D.shape[0])

    def to(self, device) -> "Scene":
        f = lambda t: None if t is None else t.to(device)
        return Scene(f(self.means3D), f(self.opacities), f(self.shs), f(self.scales), f(self.rotations),
                     self.sh_degree, self.camera.to(device), f(self.target), f(self.bg), dict(self.meta))


def _unit_quats(rng: np.random.Generator, n: int) -> np.ndarray:
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q


def _sh3(rng: np.random.Generator, n: int, degree: int = 3) -> np.ndarray:
    m = (degree + 1) ** 2
    sh = np.empty((n, m, 3))
    sh[:, 0, :] = rng.normal(0.0, 0.5, (n, 3))
    if m > 1:
        sh[:, 1:, :] = rng.normal(0.0, 0.05, (n, m - 1, 3))
    return sh


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _t(a) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))


def scene_small(n: int = 16384, width: int = 256, height: int = 256, seed: int = 0, sh_degree: int = 3) -> Scene:
    """Config-0 shape: means x,y ~ U[-1,1], z ~ U[2,6]; fx = fy = width; SH degree 3
    (DC ~ N(0,0.5), higher bands ~ N(0,0.05)); log-scales ~ N(-3.5,0.5); uniform unit
    quaternions; opacity logits ~ N(0,1); black background; target ~ U[0,1]."""
    rng = np.random.default_rng(seed)
    means = np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(2, 6, n)], axis=1)
    sh = _sh3(rng, n, sh_degree)
    scales = np.exp(rng.normal(-3.5, 0.5, (n, 3)))
    rots = _unit_quats(rng, n)
    opac = _sigmoid(rng.normal(0.0, 1.0, (n, 1)))
    target = rng.uniform(0.0, 1.0, (3, height, width))
    cam = make_camera(width, height, float(width), float(width))
    return Scene(_t(means), _t(opac), _t(sh), _t(scales), _t(rots), sh_degree, cam, _t(target),
                 meta={"workload": f"{n} SH{sh_degree} Gaussians, {width}x{height}", "seed": seed})


def scene_large(n: int = 1_000_000, width: int = 1920, height: int = 1080, seed: int = 1, sh_degree: int = 3) -> Scene:
    """Config-1 shape: means ~ N(0, 2 I) + (0,0,8) with z clipped above 0.2; fx = fy =
    1400; SH degree 3 as above; log-scales ~ N(-4.5,1.0); random unit quaternions;
    opacity logits ~ N(-1,1.5); seeded random target."""
    rng = np.random.default_rng(seed)
    means = rng.normal(0.0, math.sqrt(2.0), (n, 3)) + np.array([0.0, 0.0, 8.0])
    means[:, 2] = np.maximum(means[:, 2], 0.21)
    sh = _sh3(rng, n, sh_degree)
    scales = np.exp(rng.normal(-4.5, 1.0, (n, 3)))
    rots = _unit_quats(rng, n)
    opac = _sigmoid(rng.normal(-1.0, 1.5, (n, 1)))
    target = rng.uniform(0.0, 1.0, (3, height, width))
    cam = make_camera(width, height, 1400.0, 1400.0)
    return Scene(_t(means), _t(opac), _t(sh), _t(scales), _t(rots), sh_degree, cam, _t(target),
                 meta={"workload": f"{n} SH{sh_degree} Gaussians, {width}x{height}", "seed": seed})


# ---------------------------------------------------------------------------
# Pose-solve scenes (local Gaussians back-projected from a smooth depth field)
# ---------------------------------------------------------------------------

def _smooth_field(rng: np.random.Generator, u: np.ndarray, v: np.ndarray, waves: int = 8) -> np.ndarray:
    f = np.zeros_like(u, dtype=np.float64)
    for _ in range(waves):
        kx, ky = rng.uniform(-6.0, 6.0, 2)
        ph = rng.uniform(0, 2 * np.pi)
        amp = rng.uniform(0.5, 1.0)
        f += amp * np.sin(2 * np.pi * (kx * u + ky * v) + ph)
    return f


def random_pose(rng: np.random.Generator, max_deg: float = 5.0, max_trans: float = 0.1):
    """Ground-truth SE(3) offset: random axis, angle ~ U[0, max_deg], translation
    uniform in the ball of radius max_trans. Returns (R [3,3], t [3]) in float64."""
    axis = rng.standard_normal(3)
    axis /= np.linalg.norm(axis)
    ang = math.radians(rng.uniform(0.0, max_deg))
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K
    d = rng.standard_normal(3)
    d /= np.linalg.norm(d)
    t = d * max_trans * rng.uniform(0.0, 1.0) ** (1.0 / 3.0)
    return R, t


def scene_pose(width: int = 640, height: int = 360, n: int | None = None, seed: int = 2, fx: float | None = None) -> Scene:
    """Config-2 shape: a depth field = sum of 8 seeded 2D sinusoids mapped to [1,10];
    one Gaussian per pixel (or `n` Gaussians at random sub-pixel positions) back-projected
    through fx = fy = 500 * width/640 with a centred principal point; smooth-noise RGB as
    SH degree 0; isotropic scale = pixel footprint (depth/fx, widened by sqrt(pixels/n)
    when n < pixels); opacity logit 2. `meta` carries the ground-truth pose (R_gt, t_gt)."""
    rng = np.random.default_rng(seed)
    fx = 500.0 * width / 640.0 if fx is None else fx
    cx, cy = width / 2.0, height / 2.0
    if n is None:
        vv, uu = np.meshgrid(np.arange(height, dtype=np.float64), np.arange(width, dtype=np.float64), indexing="ij")
        uu = uu.reshape(-1)
        vv = vv.reshape(-1)
        widen = 1.0
    else:
        uu = rng.uniform(0.0, width, n) - 0.5
        vv = rng.uniform(0.0, height, n) - 0.5
        widen = math.sqrt(width * height / n)
    un, vn = (uu + 0.5) / width, (vv + 0.5) / height
    f = _smooth_field(rng, un, vn)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-9)
    depth = 1.0 + 9.0 * f
    x = (uu + 0.5 - cx) * depth / fx
    y = (vv + 0.5 - cy) * depth / fx
    means = np.stack([x, y, depth], axis=1)
    rgb = np.stack([_smooth_field(rng, un, vn, 4) for _ in range(3)], axis=1)
    rgb = 0.1 + 0.8 * (rgb - rgb.min(0)) / np.maximum(rgb.max(0) - rgb.min(0), 1e-9)
    sh = ((rgb - 0.5) / SH_C0)[:, None, :]
    s = depth / fx * widen
    scales = np.repeat(s[:, None], 3, axis=1)
    rots = np.zeros((means.shape[0], 4))
    rots[:, 0] = 1.0
    opac = _sigmoid(np.full((means.shape[0], 1), 2.0))
    R_gt, t_gt = random_pose(rng)
    cam = make_camera(width, height, fx, fx, cx, cy)
    return Scene(_t(means), _t(opac), _t(sh), _t(scales), _t(rots), 0, cam, None,
                 meta={"workload": f"pose solve, {means.shape[0]} SH0 Gaussians, {width}x{height}", "seed": seed,
                       "R_gt": R_gt, "t_gt": t_gt})


def batch_specs(count: int = 64, seed: int = 3):
    """Config-3 mix: `count` solves, N log-uniform in [5e4, 5e5], resolution from
    {320x180, 640x360, 960x540}. Returns a list of (width, height, n, seed)."""
    rng = np.random.default_rng(seed)
    res = [(320, 180), (640, 360), (960, 540)]
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(5e4), math.log(5e5)))))
        w, h = res[int(rng.integers(0, 3))]
        out.append((w, h, n, int(rng.integers(0, 2**31 - 1))))
    return out
