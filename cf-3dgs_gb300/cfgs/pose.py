"""CF-3DGS relative-pose solve through the rasteriser.

The reference (trainer/cf3dgs_trainer.py:261-285) optimises the pose of the local
Gaussians for 300 Adam iterations: the pose is lietorch's LieGroupParameter(SE3) set
to identity by CFGaussianModel.init_RT (scene/gaussian_model_cf.py:328-340) — a
6-vector tangent xi, retracted as exp(xi) * I — and positions move as
P[0].retr().act(xyz) (scene/gaussian_model_cf.py:123-133); covariances do not move
(:119-121). Adam(lr = rotation_lr = 1e-3, eps = 1e-15) runs on xi
(scene/gaussian_model_cf.py:303-326, arguments/__init__.py:111). The rendered image
is clamped to [0, 1] (scene/gaussian_model_cf.py:885) before the loss.

Two forms of the same solve:
- "plain": the SE(3) exponential and action written as PyTorch ops (lietorch is not
  available; same tangent parametrisation, ordering (rho, phi)) with autograd, and
  torch.optim.Adam — the reference's structure;
- "fused": PoseApply (cfgs_pose_apply forward, cfgs_pose_grad backward: dL/dmeans ->
  dL/dxi in one reduction kernel, no per-Gaussian Jacobians) and the Adam step as one
  kernel (cfgs_pose_adam).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import native, raster


# ---------------------------------------------------------------------------
# SE(3) in PyTorch (the plain path)
# ---------------------------------------------------------------------------
def _hat(w: torch.Tensor) -> torch.Tensor:
    z = torch.zeros((), dtype=w.dtype, device=w.device)
    return torch.stack([torch.stack([z, -w[2], w[1]]), torch.stack([w[2], z, -w[0]]),
                        torch.stack([-w[1], w[0], z])])


def so3_coeffs(th2: torch.Tensor):
    """(sin th / th, (1 - cos th)/th^2, (th - sin th)/th^3), with series near 0."""
    small = th2 < 1e-8
    th2s = torch.where(small, torch.ones_like(th2), th2)
    th = torch.sqrt(th2s)
    a = torch.where(small, 1 - th2 / 6, torch.sin(th) / th)
    b = torch.where(small, 0.5 - th2 / 24, (1 - torch.cos(th)) / th2s)
    c = torch.where(small, 1.0 / 6 - th2 / 120, (th - torch.sin(th)) / (th2s * th))
    return a, b, c


def se3_exp(xi: torch.Tensor):
    """exp of the tangent xi = (rho, phi): R = exp(phi^), t = J_l(phi) rho."""
    rho, phi = xi[:3], xi[3:]
    P = _hat(phi)
    P2 = P @ P
    a, b, c = so3_coeffs((phi * phi).sum())
    eye = torch.eye(3, dtype=xi.dtype, device=xi.device)
    R = eye + a * P + b * P2
    Jl = eye + b * P + c * P2
    return R, Jl @ rho


def se3_log_np(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Inverse of se3_exp in float64 numpy (for ground-truth tangents)."""
    cos = np.clip((np.trace(R) - 1) / 2, -1.0, 1.0)
    th = math.acos(cos)
    if th < 1e-8:
        phi = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2
    else:
        phi = th / (2 * math.sin(th)) * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    P = np.array([[0, -phi[2], phi[1]], [phi[2], 0, -phi[0]], [-phi[1], phi[0], 0]])
    th2 = float(phi @ phi)
    if th2 < 1e-12:
        b, c = 0.5, 1.0 / 6
    else:
        th = math.sqrt(th2)
        b, c = (1 - math.cos(th)) / th2, (th - math.sin(th)) / (th2 * th)
    Jl = np.eye(3) + b * P + c * P @ P
    rho = np.linalg.solve(Jl, t)
    return np.concatenate([rho, phi])


def pose_error(xi_a: np.ndarray, xi_b: np.ndarray):
    """(rotation angle between the two poses in degrees, translation distance)."""
    Ra, ta = (x.numpy() for x in se3_exp(torch.tensor(xi_a, dtype=torch.float64)))
    Rb, tb = (x.numpy() for x in se3_exp(torch.tensor(xi_b, dtype=torch.float64)))
    cos = np.clip((np.trace(Ra.T @ Rb) - 1) / 2, -1.0, 1.0)
    return math.degrees(math.acos(cos)), float(np.linalg.norm(ta - tb))


class _Act(torch.autograd.Function):
    """p' = R p + t for rotations/translations given in float64. Forward: R and t are
    rounded to the positions' dtype and each position is ((R0 x + R1 y) + R2 z) + t,
    one rounding per operation (the order the cfgs_pose_apply kernel uses, so both
    paths place the Gaussians identically). Backward: dL/dR = sum g p^T and
    dL/dt = sum g, reduced in float64."""

    @staticmethod
    def forward(ctx, R64, t64, xyz):
        R, t = R64.to(xyz.dtype), t64.to(xyz.dtype)
        x, y, z = xyz[:, 0:1], xyz[:, 1:2], xyz[:, 2:3]
        ctx.save_for_backward(xyz)
        return ((R[:, 0][None] * x + R[:, 1][None] * y) + R[:, 2][None] * z) + t[None]

    @staticmethod
    def backward(ctx, g):
        (xyz,) = ctx.saved_tensors
        g64 = g.double()
        return g64.t() @ xyz.double(), g64.sum(0), None


def apply_pose_torch(xi: torch.Tensor, xyz: torch.Tensor, cov6: torch.Tensor | None = None):
    """exp(xi).act(xyz) with autograd (the plain path). The exponential and the
    gradient reductions run in float64; the positions are float32 (see _Act)."""
    R64, t64 = se3_exp(xi.double())
    means = _Act.apply(R64, t64, xyz)
    R = R64.to(xyz.dtype)
    if cov6 is None:
        return means, None
    S = torch.stack([cov6[:, 0], cov6[:, 1], cov6[:, 2], cov6[:, 1], cov6[:, 3], cov6[:, 4], cov6[:, 2],
                     cov6[:, 4], cov6[:, 5]], 1).reshape(-1, 3, 3)
    Sr = R @ S @ R.t()
    return means, torch.stack([Sr[:, 0, 0], Sr[:, 0, 1], Sr[:, 0, 2], Sr[:, 1, 1], Sr[:, 1, 2], Sr[:, 2, 2]], 1)


# ---------------------------------------------------------------------------
# fused kernels behind autograd
# ---------------------------------------------------------------------------
class PoseApply(torch.autograd.Function):
    """means = exp(xi).act(xyz) [and cov' = R cov R^T]; backward: dL/dxi by the fused
    cfgs_pose_grad reduction (xyz and cov get no gradient: the pose solve fixes them)."""

    @staticmethod
    def forward(ctx, xi, xyz, cov6=None):
        lib = native.load()
        xi_c = xi.detach().float().contiguous()
        xyz_c = xyz.detach().float().contiguous()
        n = xyz_c.shape[0]
        means = torch.empty_like(xyz_c)
        cov_out = None
        cov_in = None
        if cov6 is not None:
            cov_in = cov6.detach().float().contiguous()
            cov_out = torch.empty_like(cov_in)
        st = torch.cuda.current_stream(xyz_c.device).cuda_stream
        native.check(lib.cfgs_pose_apply(n, xi_c.data_ptr(), xyz_c.data_ptr(),
                                         cov_in.data_ptr() if cov_in is not None else None, means.data_ptr(),
                                         cov_out.data_ptr() if cov_out is not None else None, st), "cfgs_pose_apply")
        ctx.save_for_backward(xi_c, xyz_c, cov_out if cov_out is not None else torch.empty(0))
        ctx.has_cov = cov6 is not None
        if cov6 is None:
            return means
        return means, cov_out

    @staticmethod
    def backward(ctx, g_means, g_cov=None):
        lib = native.load()
        xi_c, xyz_c, cov_rot = ctx.saved_tensors
        n = xyz_c.shape[0]
        dev = xyz_c.device
        g_means = (torch.zeros_like(xyz_c) if g_means is None else g_means).float().contiguous()
        use_cov = ctx.has_cov and g_cov is not None
        g_cov_c = g_cov.float().contiguous() if use_cov else None
        scratch = torch.empty(lib.cfgs_pose_scratch_bytes(n), dtype=torch.uint8, device=dev)
        out = torch.empty(6, dtype=torch.float32, device=dev)
        st = torch.cuda.current_stream(dev).cuda_stream
        native.check(lib.cfgs_pose_grad(n, xi_c.data_ptr(), xyz_c.data_ptr(), g_means.data_ptr(),
                                        cov_rot.data_ptr() if use_cov else None,
                                        g_cov_c.data_ptr() if use_cov else None, scratch.data_ptr(),
                                        out.data_ptr(), st), "cfgs_pose_grad")
        if ctx.has_cov:
            return out, None, None
        return out, None


def pose_apply(xi, xyz, cov6=None):
    if cov6 is None:
        return PoseApply.apply(xi, xyz)
    return PoseApply.apply(xi, xyz, cov6)


class FusedAdam:
    """torch.optim.Adam (no weight decay) on one or more 6-vectors (xi [6] or [S,6]),
    one kernel per step for all of them; moments and step counts stay on the device."""

    def __init__(self, xi: torch.Tensor, lr=1e-3, betas=(0.9, 0.999), eps=1e-15):
        self.xi = xi
        self.count = xi.numel() // 6
        self.lr, self.b1, self.b2, self.eps = float(lr), float(betas[0]), float(betas[1]), float(eps)
        self.state = torch.zeros(self.count, 16, dtype=torch.float32, device=xi.device)

    def step(self, grad: torch.Tensor):
        lib = native.load()
        st = torch.cuda.current_stream(self.xi.device).cuda_stream
        native.check(lib.cfgs_pose_adam(self.count, self.xi.data_ptr(), grad.contiguous().data_ptr(),
                                        self.state.data_ptr(), self.lr, self.b1, self.b2, self.eps, st),
                     "cfgs_pose_adam")


# ---------------------------------------------------------------------------
# the solve
# ---------------------------------------------------------------------------
@dataclass
class PoseProblem:
    """Device-resident inputs of one relative-pose solve."""
    xyz: torch.Tensor         # [N,3] local Gaussians (frame t-1)
    opacities: torch.Tensor   # [N,1]
    shs: torch.Tensor         # [N,M,3]
    scales: torch.Tensor      # [N,3]
    rotations: torch.Tensor   # [N,4]
    sh_degree: int
    settings: object          # GaussianRasterizationSettings
    target: torch.Tensor      # [3,H,W] frame t
    xi_gt: np.ndarray | None = None


def make_problem(scene, device="cuda") -> PoseProblem:
    """Builds the device problem of a pose scene; the target is the same Gaussians
    rendered at the scene's ground-truth pose."""
    import diff_gaussian_rasterization as dgr
    s = scene.to(device)
    cam = s.camera
    rs = dgr.GaussianRasterizationSettings(cam.height, cam.width, cam.tanfovx, cam.tanfovy, s.bg, 1.0,
                                           cam.viewmatrix, cam.projmatrix, s.sh_degree, cam.campos, False, False)
    xi_gt = se3_log_np(scene.meta["R_gt"], scene.meta["t_gt"])
    prob = PoseProblem(s.means3D, s.opacities, s.shs, s.scales, s.rotations, s.sh_degree, rs, None, xi_gt)
    with torch.no_grad():
        means, _ = apply_pose_torch(torch.tensor(xi_gt, dtype=torch.float32, device=device), s.means3D)
        img = render(prob, means)
    prob.target = img.detach().clamp(0, 1).contiguous()
    return prob


def render(prob: PoseProblem, means: torch.Tensor, cov6: torch.Tensor | None = None) -> torch.Tensor:
    import diff_gaussian_rasterization as dgr
    means2D = torch.zeros_like(means)
    r = dgr.GaussianRasterizer(prob.settings)
    if cov6 is None:
        color, radii, depth, alpha = r(means3D=means, means2D=means2D, opacities=prob.opacities, shs=prob.shs,
                                       scales=prob.scales, rotations=prob.rotations)
    else:
        color, radii, depth, alpha = r(means3D=means, means2D=means2D, opacities=prob.opacities, shs=prob.shs,
                                       cov3D_precomp=cov6)
    return color


def l1(img: torch.Tensor, target: torch.Tensor, fused: bool = False) -> torch.Tensor:
    """RGB L1 of the clamped render (trainer/losses.py:98-136 with lambda_dssim = 0):
    PyTorch operations on the plain path, the fused L1 kernels on the fused path."""
    if fused:
        from .loss import l1_loss
        return l1_loss(img, target, clamp=True)
    return (img.clamp(0, 1) - target).abs().mean()


def ssim_torch(img1: torch.Tensor, img2: torch.Tensor) -> torch.Tensor:
    """The reference's SSIM in PyTorch (utils/loss_utils.py:23-58: 11x11 Gaussian window,
    sigma 1.5, depthwise conv2d with zero padding 5): the plain path's SSIM."""
    import torch.nn.functional as F
    C = img1.shape[-3]
    w1 = torch.exp(-((torch.arange(11, dtype=torch.float64) - 5) ** 2) / (2 * 1.5 ** 2))
    w1 = (w1 / w1.sum()).to(img1)
    win = (w1[:, None] @ w1[None, :]).expand(C, 1, 11, 11).contiguous()
    x, y = img1.reshape(1, C, *img1.shape[-2:]), img2.reshape(1, C, *img2.shape[-2:])
    mu1, mu2 = F.conv2d(x, win, padding=5, groups=C), F.conv2d(y, win, padding=5, groups=C)
    s11 = F.conv2d(x * x, win, padding=5, groups=C) - mu1 * mu1
    s22 = F.conv2d(y * y, win, padding=5, groups=C) - mu2 * mu2
    s12 = F.conv2d(x * y, win, padding=5, groups=C) - mu1 * mu2
    c1, c2 = 0.01 ** 2, 0.03 ** 2
    return (((2 * mu1 * mu2 + c1) * (2 * s12 + c2)) / ((mu1 * mu1 + mu2 * mu2 + c1) * (s11 + s22 + c2))).mean()


def photometric_loss(img: torch.Tensor, target: torch.Tensor, lambda_dssim: float, fused: bool) -> torch.Tensor:
    """(1 - lambda) L1 + lambda (1 - SSIM) of the clamped render (trainer/losses.py:98-136;
    CF-3DGS uses lambda_dssim = 0.2). lambda 0 is the RGB L1 alone."""
    if lambda_dssim == 0.0:
        return l1(img, target, fused)
    c = img.clamp(0, 1)
    if fused:
        from .ssim import ssim
        return (1.0 - lambda_dssim) * l1(img, target, fused=True) + lambda_dssim * (1.0 - ssim(c, target))
    return (1.0 - lambda_dssim) * (c - target).abs().mean() + lambda_dssim * (1.0 - ssim_torch(c, target))


def solve(prob: PoseProblem, iters: int = 300, lr: float = 1e-3, mode: str = "fused", record: bool = False,
          lambda_dssim: float = 0.0):
    """Runs the pose solve; returns (xi [6] float64 numpy, losses list if record).
    lambda_dssim > 0 adds the SSIM term of the reference's loss (PyTorch SSIM on the
    plain path, the fused SSIM kernels on the fused path)."""
    dev = prob.xyz.device
    losses = []
    if mode == "plain":
        xi = torch.zeros(6, dtype=torch.float32, device=dev, requires_grad=True)
        opt = torch.optim.Adam([xi], lr=lr, eps=1e-15)
        for _ in range(iters):
            means, _ = apply_pose_torch(xi, prob.xyz)
            loss = photometric_loss(render(prob, means), prob.target, lambda_dssim, fused=False)
            loss.backward()
            opt.step()
            opt.zero_grad(set_to_none=True)
            if record:
                losses.append(float(loss.detach()))
        return xi.detach().double().cpu().numpy(), losses
    if mode == "fused":
        xi = torch.zeros(6, dtype=torch.float32, device=dev)
        opt = FusedAdam(xi, lr=lr)
        for _ in range(iters):
            xi_leaf = xi.detach().requires_grad_(True)
            means = pose_apply(xi_leaf, prob.xyz)
            loss = photometric_loss(render(prob, means), prob.target, lambda_dssim, fused=True)
            loss.backward()
            opt.step(xi_leaf.grad)
            if record:
                losses.append(float(loss.detach()))
        return xi.detach().double().cpu().numpy(), losses
    raise ValueError(mode)


def time_solves(prob: PoseProblem, mode: str, count: int = 3, iters: int = 300):
    """Wall-clock solves/s and per-solve latencies of `count` back-to-back solves."""
    lat = []
    for _ in range(count):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solve(prob, iters=iters, mode=mode)
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t0)
    return count / sum(lat), lat
