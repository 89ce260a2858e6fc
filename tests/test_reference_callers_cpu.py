"""The reference's own render callers, unchanged, through this package's drop-in
`diff_gaussian_rasterization` (CPU: the drop-in's two native calls are served by the C
oracle; see reference_callers.py).

CF3DGS_Render.render (scene/gaussian_model_cf.py:777-910) and gaussian_renderer.render
(gaussian_renderer/__init__.py:19-113) build the settings, call GaussianRasterizer with
keyword arguments, unpack the 4-tuple, clamp the image (the former) and hand back the
screen-space points whose .grad add_densification_stats reads
(scene/gaussian_model_cf.py:716-719). Checked: each output and every gradient equals the
oracle's for the tensors the callers passed, across the callers' switches
(compute_cov3D_python, convert_SHs_python); and the settings the callers built are the
12-field NamedTuple of the drop-in.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import reference_callers as RC

pytestmark = pytest.mark.skipif(not RC.available(), reason="reference tree not present")


@pytest.fixture()
def oracle_raster(monkeypatch):
    from cfgs import raster
    o = RC.OracleRaster()
    monkeypatch.setattr(raster, "forward", o.forward)
    monkeypatch.setattr(raster, "backward", o.backward)
    return o


def _scene():
    from cfgs import scenes
    sc = scenes.scene_small(n=1500, width=64, height=48, seed=13)
    return sc


def _expected(call, image_grad, depth_grad=None, alpha_grad=None):
    from oracle.c_oracle import Oracle
    rs, x = call["settings"], call["inputs"]
    o = Oracle(rs["image_width"], rs["image_height"], rs["tanfovx"], rs["tanfovy"], rs["bg"], rs["scale_modifier"],
               rs["viewmatrix"], rs["projmatrix"], rs["sh_degree"], rs["campos"], x["means3D"], x["opacities"],
               shs=x["shs"], colors_precomp=x["colors_precomp"], scales=x["scales"], rotations=x["rotations"],
               cov3D_precomp=x["cov3D_precomp"]).forward()
    return o, o.backward(image_grad, depth_grad, alpha_grad)


@pytest.mark.parametrize("cov_python", [False, True])
@pytest.mark.parametrize("shs_python", [False, True])
def test_cf3dgs_render_through_dropin(oracle_raster, cov_python, shs_python):
    sc = _scene()
    with RC.reference_modules() as (gm, gr):
        rend = gm.CF3DGS_Render(sh_degree=3, white_background=False)
        RC.load_scene_into(rend.gaussians, sc)
        cam = RC.Camera(sc.camera)
        out = rend.render(cam, compute_cov3D_python=cov_python, convert_SHs_python=shs_python)
        assert set(out) == {"image", "depth", "alpha", "viewspace_points", "visibility_filter", "radii"}
        w = torch.linspace(-1.0, 1.0, out["image"].numel()).reshape(out["image"].shape)
        loss = (out["image"] * w).sum() + 1e-3 * out["depth"].sum() - 1e-3 * out["alpha"].sum()
        loss.backward()
    call = oracle_raster.calls[-1]
    from diff_gaussian_rasterization import GaussianRasterizationSettings
    assert list(call["settings"]) == list(GaussianRasterizationSettings._fields) and len(call["settings"]) == 12
    assert (call["inputs"]["cov3D_precomp"] is not None) == cov_python
    assert (call["inputs"]["shs"] is None) == (shs_python and not rend.view_dependent)
    gi = call["grads_in"]
    o, g = _expected(call, gi["color"].numpy(), gi["depth"].numpy(), gi["alpha"].numpy())
    # the caller clamps the image to [0, 1] (scene/gaussian_model_cf.py:885)
    assert torch.equal(out["image"], torch.from_numpy(o.color).clamp(0, 1))
    assert torch.equal(out["radii"], torch.from_numpy(o.radii))
    assert torch.equal(out["depth"], torch.from_numpy(o.depth)) and torch.equal(out["alpha"], torch.from_numpy(o.alpha))
    assert torch.equal(out["visibility_filter"], torch.from_numpy(o.radii > 0))
    # the image gradient that reached the rasteriser went through the clamp
    inside = ((torch.from_numpy(o.color) >= 0) & (torch.from_numpy(o.color) <= 1)).float()
    assert torch.equal(gi["color"], w * inside)
    # screen-space gradients land on the caller's viewspace points
    np.testing.assert_array_equal(out["viewspace_points"].grad.numpy(), g["means2D"])
    if not cov_python:
        np.testing.assert_array_equal(rend.gaussians._xyz.grad.numpy(), g["means3D"])
    if not shs_python:
        sh = torch.cat([rend.gaussians._features_dc.grad, rend.gaussians._features_rest.grad], 1).numpy()
        np.testing.assert_array_equal(sh, g["sh"])


@pytest.mark.parametrize("cov_python,shs_python", [(False, False), (True, True)])
def test_gaussian_renderer_through_dropin(oracle_raster, cov_python, shs_python):
    sc = _scene()
    with RC.reference_modules() as (gm, gr):
        model = gm.CFGaussianModel(3)
        RC.load_scene_into(model, sc)
        bg = torch.tensor([0.2, 0.4, 0.6])
        out = gr.render(RC.Camera(sc.camera), model, RC.Pipe(cov_python, shs_python), bg)
        assert set(out) == {"render", "viewspace_points", "visibility_filter", "radii", "depth", "alpha"}
        w = torch.linspace(1.0, -1.0, out["render"].numel()).reshape(out["render"].shape)
        (out["render"] * w).sum().backward()
    call = oracle_raster.calls[-1]
    assert torch.equal(call["settings"]["bg"], bg)
    o, g = _expected(call, call["grads_in"]["color"].numpy())
    assert call["grads_in"]["depth"] is None and call["grads_in"]["alpha"] is None  # unused outputs: no gradient
    assert torch.equal(out["render"], torch.from_numpy(o.color))  # this caller does not clamp
    assert torch.equal(out["radii"], torch.from_numpy(o.radii))
    np.testing.assert_array_equal(out["viewspace_points"].grad.numpy(), g["means2D"])
    if not cov_python:
        np.testing.assert_array_equal(model._xyz.grad.numpy(), g["means3D"])


def test_recorded_calls_match_committed_fixture(oracle_raster):
    """The fixture tests/golden/reference_callers.npz (made by
    tests/golden/make_reference_callers.py from these callers) still holds what the
    callers pass to the rasteriser, so the GPU replay of it tests the current callers."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "reference_callers.npz")
    fx = np.load(path)
    sc = _scene()
    with RC.reference_modules() as (gm, gr):
        rend = gm.CF3DGS_Render(sh_degree=3, white_background=False)
        RC.load_scene_into(rend.gaussians, sc)
        rend.render(RC.Camera(sc.camera))
    call = oracle_raster.calls[-1]
    for k in ("means3D", "opacities", "shs", "scales", "rotations"):
        np.testing.assert_array_equal(call["inputs"][k].numpy(), fx[f"in_{k}"], err_msg=k)
    for k in ("viewmatrix", "projmatrix", "campos", "bg"):
        np.testing.assert_array_equal(call["settings"][k].numpy(), fx[f"set_{k}"], err_msg=k)
    assert float(call["settings"]["tanfovx"]) == float(fx["set_tanfovx"])
