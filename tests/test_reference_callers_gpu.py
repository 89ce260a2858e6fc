"""Replay, on the GPU, of the rasteriser call the reference's CF3DGS_Render.render makes
(scene/gaussian_model_cf.py:777-910), recorded in tests/golden/reference_callers.npz by
tests/golden/make_reference_callers.py (the CPU test test_reference_callers_cpu.py runs
the caller itself, unchanged, through this drop-in package).

The same settings and tensors go through diff_gaussian_rasterization on the CUDA path:
the image, depth, alpha and radii equal what the caller received (bit for bit), the
caller's clamp of the image gives its output, and the screen-space and 3D-mean
gradients for the caller's image gradient agree with the oracle's within 1e-4 relative
or the float32 rounding bound (oracle.error_bound).
"""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from helpers import assert_grad_bounded, bits

pytestmark = pytest.mark.gpu
DEV = "cuda"
FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "reference_callers.npz")


def test_replay_of_cf3dgs_render_call():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as dgr
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds
    fx = np.load(FIXTURE)
    t = lambda k: torch.from_numpy(fx[k]).to(DEV)
    rs = dgr.GaussianRasterizationSettings(
        image_height=int(fx["set_image_height"]), image_width=int(fx["set_image_width"]),
        tanfovx=float(fx["set_tanfovx"]), tanfovy=float(fx["set_tanfovy"]), bg=t("set_bg"),
        scale_modifier=float(fx["set_scale_modifier"]), viewmatrix=t("set_viewmatrix"),
        projmatrix=t("set_projmatrix"), sh_degree=int(fx["set_sh_degree"]), campos=t("set_campos"),
        prefiltered=bool(fx["set_prefiltered"]), debug=bool(fx["set_debug"]))
    means3D = t("in_means3D").requires_grad_(True)
    means2D = torch.zeros_like(means3D, requires_grad=True)
    opac, shs = t("in_opacities").requires_grad_(True), t("in_shs").requires_grad_(True)
    scales, rots = t("in_scales").requires_grad_(True), t("in_rotations").requires_grad_(True)
    color, radii, depth, alpha = dgr.GaussianRasterizer(rs)(means3D=means3D, means2D=means2D, shs=shs,
                                                            colors_precomp=None, opacities=opac, scales=scales,
                                                            rotations=rots, cov3D_precomp=None)
    image = color.clamp(0, 1)  # the caller's clamp, scene/gaussian_model_cf.py:885
    np.testing.assert_array_equal(bits(image.detach().cpu().numpy()), bits(fx["out_image"]))
    np.testing.assert_array_equal(radii.cpu().numpy(), fx["out_radii"])
    np.testing.assert_array_equal(bits(depth.detach().cpu().numpy()), bits(fx["out_depth"]))
    np.testing.assert_array_equal(bits(alpha.detach().cpu().numpy()), bits(fx["out_alpha"]))
    color.backward(t("grad_color"))
    torch.cuda.synchronize()
    ref = Oracle(int(fx["set_image_width"]), int(fx["set_image_height"]), float(fx["set_tanfovx"]),
                 float(fx["set_tanfovy"]), fx["set_bg"], float(fx["set_scale_modifier"]), fx["set_viewmatrix"],
                 fx["set_projmatrix"], int(fx["set_sh_degree"]), fx["set_campos"], fx["in_means3D"],
                 fx["in_opacities"], shs=fx["in_shs"], scales=fx["in_scales"], rotations=fx["in_rotations"]).forward()
    want = ref.backward(fx["grad_color"], magnitudes=True)
    bound = backward_bounds(ref)
    # what the caller read: viewspace_points.grad and the means' gradient
    np.testing.assert_array_equal(want["means2D"], fx["out_viewspace_grad"])
    np.testing.assert_array_equal(want["means3D"], fx["out_xyz_grad"])
    assert_grad_bounded("viewspace_points", means2D.grad.cpu(), fx["out_viewspace_grad"], bound["means2D"])
    assert_grad_bounded("means3D", means3D.grad.cpu(), fx["out_xyz_grad"], bound["means3D"])
    assert_grad_bounded("shs", shs.grad.cpu(), want["sh"], bound["sh"])
    assert_grad_bounded("opacities", opac.grad.cpu(), want["opacity"], bound["opacity"])
    assert_grad_bounded("scales", scales.grad.cpu(), want["scales"], bound["scales"])
    assert_grad_bounded("rotations", rots.grad.cpu(), want["rotations"], bound["rotations"])
