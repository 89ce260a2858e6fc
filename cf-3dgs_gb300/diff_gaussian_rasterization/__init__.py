"""GB300 drop-in for the `diff_gaussian_rasterization` package used by CF-3DGS.

Same public surface as the package the reference imports at
scene/gaussian_model_cf.py:28-31, gaussian_renderer/__init__.py:12 and
scene/gaussian_model.py:27-30:

- ``GaussianRasterizationSettings``: NamedTuple with the 12 fields in the order the
  reference builds it (scene/gaussian_model_cf.py:811-824);
- ``GaussianRasterizer(raster_settings)``: ``forward(means3D, means2D, opacities,
  shs=None, colors_precomp=None, scales=None, rotations=None, cov3D_precomp=None)``
  returning ``(color [3,H,W], radii [N] int32, depth [1,H,W], alpha [1,H,W])`` (the
  4-tuple unpacked at scene/gaussian_model_cf.py:883-884), and
  ``markVisible(positions) -> bool[N]``;
- ``rasterize_gaussians(...)``: the functional form behind the module.

All computation runs in libcfgs.so (hand-written sm_103a kernels) through its C ABI.
"""
from __future__ import annotations

import os
import sys
from typing import NamedTuple

import torch
import torch.nn as nn

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _PKG_ROOT not in sys.path:
    sys.path.insert(0, _PKG_ROOT)

from cfgs import raster as _raster  # noqa: E402
from cfgs import native as _native  # noqa: E402

_native.load()  # fail at import when the native library is unavailable


class GaussianRasterizationSettings(NamedTuple):
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    sh_degree: int
    campos: torch.Tensor
    prefiltered: bool
    debug: bool


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                        raster_settings):
    return _raster.RasterizeGaussiansFn.apply(means3D, means2D, sh, colors_precomp, opacities, scales, rotations,
                                              cov3Ds_precomp, raster_settings)


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings: GaussianRasterizationSettings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions: torch.Tensor) -> torch.Tensor:
        """Boolean mask of the points in front of the near plane (view z > 0.2)."""
        with torch.no_grad():
            rs = self.raster_settings
            return _raster.mark_visible(positions, rs.viewmatrix, rs.projmatrix)

    def forward(self, means3D, means2D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                cov3D_precomp=None):
        rs = self.raster_settings
        if (shs is None) == (colors_precomp is None):
            raise Exception("Please provide exactly one of either SHs or precomputed colors!")
        if ((scales is None or rotations is None) and cov3D_precomp is None) or (
                (scales is not None or rotations is not None) and cov3D_precomp is not None):
            raise Exception("Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!")
        empty = torch.Tensor([])
        if shs is None:
            shs = empty
        if colors_precomp is None:
            colors_precomp = empty
        if scales is None:
            scales = empty
        if rotations is None:
            rotations = empty
        if cov3D_precomp is None:
            cov3D_precomp = empty
        return rasterize_gaussians(means3D, means2D, shs, colors_precomp, opacities, scales, rotations,
                                   cov3D_precomp, rs)


__all__ = ["GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians"]
