"""The oracle pinned against golden vectors produced by the reference's own Python
(tests/golden/make_golden.py): SH evaluation (utils/sh_utils.py), the covariance from
scale and quaternion (utils/general_utils.py), and the intrinsics camera
(scene/cameras.py + utils/graphics_utils.py)."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_math.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_torch_oracle_sh_matches_reference(g, deg):
    from oracle import torch_oracle as TO
    d = torch.tensor(g["sh_dirs"], dtype=torch.float64)
    c = torch.tensor(g["sh_coeffs"], dtype=torch.float64)
    B = TO.sh_basis(deg, d)
    m = (deg + 1) ** 2
    col = torch.clamp_min((B[:, :, None] * c[:, :m, :]).sum(1) + 0.5, 0.0).numpy()
    np.testing.assert_allclose(col, g[f"sh_color_deg{deg}"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_c_oracle_sh_colour_matches_reference(g, deg):
    """The C oracle's in-preprocess SH colour (what the GPU kernel reproduces bit for
    bit) for Gaussians placed along the golden directions, in front of a 90-degree
    camera at the origin."""
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    d = g["sh_dirs"].astype(np.float64)
    means = (4.0 * d).astype(np.float32)
    n = len(d)
    cam = scenes.make_camera(64, 64, 32.0, 32.0)
    o = Oracle(64, 64, cam.tanfovx, cam.tanfovy, np.zeros(3, np.float32), 1.0, cam.viewmatrix, cam.projmatrix, deg,
               cam.campos, means, np.full((n, 1), 0.5, np.float32), shs=g["sh_coeffs"],
               scales=np.full((n, 3), 0.05, np.float32), rotations=np.tile([1, 0, 0, 0], (n, 1)).astype(np.float32))
    o.forward()
    vis = o.radii > 0
    assert vis.sum() >= 8
    np.testing.assert_allclose(o.rgbd[vis, :3], g[f"sh_color_deg{deg}"][vis], rtol=0, atol=2e-6)


@pytest.mark.parametrize("mod", [1.0, 0.7])
def test_covariance_matches_reference(g, mod):
    from oracle import torch_oracle as TO
    cov = TO.cov3d(torch.tensor(g["cov_scales"], dtype=torch.float64),
                   torch.tensor(g["cov_rotations"], dtype=torch.float64), mod).numpy()
    want = g[f"cov3d_mod{mod}"]  # the reference computes it in float32
    np.testing.assert_allclose(cov, want, rtol=0, atol=2e-6 * np.abs(want).max())


@pytest.mark.parametrize("i", [0, 1, 2, 3])
def test_camera_matches_reference(g, i):
    from cfgs import scenes
    W, H, fx, fy, cx, cy = g[f"cam{i}_intr"]
    cam = scenes.make_camera(int(W), int(H), float(fx), float(fy), float(cx), float(cy), R=g[f"cam{i}_R"],
                             T=g[f"cam{i}_T"])
    np.testing.assert_allclose(cam.viewmatrix.numpy(), g[f"cam{i}_view"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(cam.projmatrix.numpy(), g[f"cam{i}_full"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(cam.campos.numpy(), g[f"cam{i}_center"], rtol=0, atol=1e-5)
    np.testing.assert_allclose([cam.tanfovx, cam.tanfovy], g[f"cam{i}_tanfov"], rtol=1e-7)


def test_ssim_oracle_matches_reference():
    """oracle/ssim_oracle.py against the reference's utils/loss_utils.py ssim (value and
    autograd gradient, float64) on the golden image pairs."""
    from oracle import ssim_oracle
    g = np.load(GOLD)
    for i in range(3):
        v, grad = ssim_oracle.ssim(g[f"ssim{i}_img1"], g[f"ssim{i}_img2"], with_grad=True)
        # the reference's window is rounded to float32 (utils/loss_utils.py:27-28)
        assert abs(v - float(g[f"ssim{i}_value"])) < 1e-6
        ref = g[f"ssim{i}_grad"]
        assert np.abs(grad - ref).max() <= 1e-5 * np.abs(ref).max()
