"""Makes tests/golden/reference_callers.npz: what the reference's CF3DGS_Render.render
(scene/gaussian_model_cf.py:777-910) passes to the rasteriser and what it returns, for a
seeded 1,500-Gaussian SH3 scene at 64x48, with the C oracle behind the drop-in's native
calls (tests/reference_callers.py). Run in a checkout that has the reference tree
(CFGS_REFERENCE_ROOT); the GPU test tests/test_reference_callers_gpu.py replays the
recorded call through the CUDA path.

    python tests/golden/make_reference_callers.py
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "cf-3dgs_gb300"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import reference_callers as RC  # noqa: E402


def main():
    from cfgs import raster, scenes
    if not RC.available():
        raise SystemExit("the reference tree is not present (set CFGS_REFERENCE_ROOT)")
    o = RC.OracleRaster()
    raster.forward, raster.backward = o.forward, o.backward
    sc = scenes.scene_small(n=1500, width=64, height=48, seed=13)
    with RC.reference_modules() as (gm, gr):
        rend = gm.CF3DGS_Render(sh_degree=3, white_background=False)
        RC.load_scene_into(rend.gaussians, sc)
        out = rend.render(RC.Camera(sc.camera))
        w = torch.linspace(-1.0, 1.0, out["image"].numel()).reshape(out["image"].shape)
        (out["image"] * w).sum().backward()
    call = o.calls[-1]
    fx = {f"in_{k}": v.numpy() for k, v in call["inputs"].items() if v is not None}
    for k, v in call["settings"].items():
        fx[f"set_{k}"] = v.numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
    fx["out_image"] = out["image"].detach().numpy()
    fx["out_radii"] = out["radii"].numpy()
    fx["out_depth"] = out["depth"].detach().numpy()
    fx["out_alpha"] = out["alpha"].detach().numpy()
    fx["grad_color"] = call["grads_in"]["color"].numpy()
    fx["out_viewspace_grad"] = out["viewspace_points"].grad.numpy()
    fx["out_xyz_grad"] = rend.gaussians._xyz.grad.numpy()
    np.savez_compressed(os.path.join(HERE, "reference_callers.npz"), **fx)
    print("wrote", os.path.join(HERE, "reference_callers.npz"), {k: v.shape for k, v in fx.items()})


if __name__ == "__main__":
    main()
