"""SE(3) restatement of the pose path (CPU): exp/log round trip, Rodrigues agreement,
and the left-Jacobian chain the fused kernel implements, checked by autograd."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch


def test_exp_log_round_trip_and_rodrigues():
    from cfgs import pose, scenes
    rng = np.random.default_rng(0)
    for scale in (0.0, 1e-9, 1e-4, 0.1, 1.0, 2.5):
        xi = rng.standard_normal(6) * scale
        R, t = (x.numpy() for x in pose.se3_exp(torch.tensor(xi, dtype=torch.float64)))
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12)
        phi = xi[3:]
        th = np.linalg.norm(phi)
        K = np.array([[0, -phi[2], phi[1]], [phi[2], 0, -phi[0]], [-phi[1], phi[0], 0]])
        if th > 0:
            Rr = np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * K @ K
            assert np.allclose(R, Rr, atol=1e-12)
        back = pose.se3_log_np(R, t)
        assert np.allclose(back, xi, atol=1e-9)
    Rg, tg = scenes.random_pose(np.random.default_rng(3))
    xi = pose.se3_log_np(Rg, tg)
    R, t = (x.numpy() for x in pose.se3_exp(torch.tensor(xi, dtype=torch.float64)))
    assert np.allclose(R, Rg, atol=1e-12) and np.allclose(t, tg, atol=1e-12)


def test_left_jacobian_chain_matches_autograd():
    """dL/dxi = J(xi)^T (sum g, sum p' x g): the formula the fused kernel evaluates,
    checked here in float64 against autograd of exp(xi).act(p)."""
    from cfgs import pose
    g = torch.Generator().manual_seed(1)
    xi = torch.randn(6, generator=g, dtype=torch.float64) * 0.4
    p = torch.randn(100, 3, generator=g, dtype=torch.float64)
    gm = torch.randn(100, 3, generator=g, dtype=torch.float64)
    x = xi.clone().requires_grad_(True)
    m, _ = pose.apply_pose_torch(x, p)
    (m * gm).sum().backward()
    R, t = pose.se3_exp(xi)
    pp = p @ R.t() + t
    d_rho = gm.sum(0)
    d_phi = torch.cross(pp, gm, dim=1).sum(0)
    # numeric SE(3) left Jacobian: exp(xi + e) exp(xi)^-1 ~ exp(J e)
    J = torch.zeros(6, 6, dtype=torch.float64)
    h = 1e-6
    for k in range(6):
        e = torch.zeros(6, dtype=torch.float64)
        e[k] = h
        Rp, tp = pose.se3_exp(xi + e)
        Rm, tm = pose.se3_exp(xi - e)
        dR = (Rp - Rm) / (2 * h) @ R.t()
        dt = (tp - tm) / (2 * h) - dR @ t
        J[:3, k] = dt
        J[3:, k] = torch.stack([dR[2, 1], dR[0, 2], dR[1, 0]])
    want = J.t() @ torch.cat([d_rho, d_phi])
    assert torch.allclose(x.grad, want, rtol=1e-6, atol=1e-6)


def test_pose_scene_is_consistent():
    from cfgs import scenes
    sc = scenes.scene_pose(width=64, height=36, seed=1)
    assert sc.n == 64 * 36
    z = sc.means3D[:, 2]
    assert float(z.min()) >= 1.0 - 1e-5 and float(z.max()) <= 10.0 + 1e-5
    u = sc.means3D[:, 0] / z * sc.camera.fx + sc.camera.cx - 0.5
    assert torch.allclose(u.reshape(36, 64)[0], torch.arange(64, dtype=torch.float32), atol=1e-3)
    R, t = sc.meta["R_gt"], sc.meta["t_gt"]
    ang = math.degrees(math.acos(np.clip((np.trace(R) - 1) / 2, -1, 1)))
    assert 0.0 <= ang <= 5.0 + 1e-9 and np.linalg.norm(t) <= 0.1 + 1e-12
