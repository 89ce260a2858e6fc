"""The plain GPU path of the rasteriser: the published 3D Gaussian Splatting rasteriser's
structure (include/cfgs_plain.h), called the way the upstream `_C` functions are called
(`rasterize_gaussians` / `rasterize_gaussians_backward`, workspaces allocated per call
from torch's caching allocator, the instance count read back to the host before the
instance buffers are sized).

It is the GPU comparison point for the tuned path in `cfgs.raster`: same preprocess and
per-Gaussian backward kernels, same per-pixel arithmetic, but 64-bit keys with one radix
sort, one thread per pixel, and gradients accumulated with global atomic adds. Not used
by the drop-in module.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import native
from .raster import _ptr, _Timed, make_gaussians, make_settings, stream_handle

ERR_CAPACITY = 2  # CFGS_ERR_CAPACITY


@dataclass
class PlainState:
    geom: torch.Tensor
    image: torch.Tensor
    work: torch.Tensor
    capacity: int
    num_rendered: int
    radii: torch.Tensor


def _work(lib, N: int, capacity: int, W: int, H: int, dev) -> torch.Tensor:
    nbytes = int(lib.cfgs_plain_work_bytes(N, capacity, W, H))
    if nbytes == 0:
        raise RuntimeError("cfgs_plain_work_bytes: the sort's storage query failed")
    return torch.empty(nbytes, dtype=torch.uint8, device=dev)


def forward(rs, means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp, timers=None,
            capacity_hint: int = 0):
    """Preprocess, plain binning, plain compositing. Returns (color, radii, depth, alpha,
    PlainState). `capacity_hint` sizes the first workspace (instances); a count above it
    grows the workspace and bins again, as upstream resizes its buffers."""
    lib = native.load()
    dev = means3D.device
    if dev.type != "cuda":
        raise RuntimeError("the plain rasteriser needs CUDA tensors; got " + str(dev))
    keep: list = []
    s = make_settings(rs, keep)
    g = make_gaussians(means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp)
    N = g.num_gaussians
    H, W = s.image_height, s.image_width
    st = stream_handle(dev)
    geom = torch.empty(lib.cfgs_geom_bytes(N), dtype=torch.uint8, device=dev)
    image = torch.empty(lib.cfgs_image_bytes(W, H), dtype=torch.uint8, device=dev)
    radii = torch.empty(N, dtype=torch.int32, device=dev)
    with _Timed(timers, "preprocess"):
        native.check(lib.cfgs_preprocess_forward(C.byref(s), C.byref(g), geom.data_ptr(), image.data_ptr(),
                                                 radii.data_ptr() if N else None, st), "cfgs_preprocess_forward")
    capacity = max(int(capacity_hint), 1)
    work = _work(lib, N, capacity, W, H, dev)
    K = C.c_int64(0)
    with _Timed(timers, "bin"):
        rc = lib.cfgs_plain_bin(C.byref(s), N, geom.data_ptr(), work.data_ptr(), capacity, C.byref(K), st)
        if rc == ERR_CAPACITY:
            capacity = int(K.value)
            work = _work(lib, N, capacity, W, H, dev)
            rc = lib.cfgs_plain_bin(C.byref(s), N, geom.data_ptr(), work.data_ptr(), capacity, C.byref(K), st)
        native.check(rc, "cfgs_plain_bin")
    color = torch.empty((3, H, W), dtype=torch.float32, device=dev)
    depth = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    alpha = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    with _Timed(timers, "composite"):
        native.check(lib.cfgs_plain_render_forward(C.byref(s), N, geom.data_ptr(), image.data_ptr(), work.data_ptr(),
                                                   capacity, color.data_ptr(), depth.data_ptr(), alpha.data_ptr(),
                                                   st), "cfgs_plain_render_forward")
    return color, radii, depth, alpha, PlainState(geom, image, work, capacity, int(K.value), radii)


def backward(rs, state: PlainState, means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp,
             grad_color, grad_depth=None, grad_alpha=None, timers=None):
    """Returns (dmeans2D, dcolors, dopacity, dmeans3D, dcov3D, dsh, dscales, drotations),
    as `cfgs.raster.backward`."""
    lib = native.load()
    dev = means3D.device
    keep: list = []
    s = make_settings(rs, keep)
    g = make_gaussians(means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp)
    N = g.num_gaussians
    st = stream_handle(dev)
    grad_color = grad_color.float().contiguous()
    grad_depth = None if grad_depth is None else grad_depth.float().contiguous()
    grad_alpha = None if grad_alpha is None else grad_alpha.float().contiguous()
    f = dict(device=dev, dtype=torch.float32)
    d_m2 = torch.empty((N, 3), **f)
    d_col = torch.empty((N, 3), **f)
    d_op = torch.empty((N, 1), **f)
    d_m3 = torch.empty((N, 3), **f)
    d_cov = torch.empty((N, 6), **f)
    d_sh = torch.empty_like(shs) if shs is not None else None
    d_sc = torch.empty((N, 3), **f) if cov3D_precomp is None else None
    d_rot = torch.empty((N, 4), **f) if cov3D_precomp is None else None
    gr = native.Gradients()
    gr.dL_dmeans2D = _ptr(d_m2)
    gr.dL_dcolors = _ptr(d_col)
    gr.dL_dopacity = _ptr(d_op)
    gr.dL_dmeans3D = _ptr(d_m3)
    gr.dL_dcov3D = _ptr(d_cov)
    gr.dL_dsh = _ptr(d_sh)
    gr.dL_dscales = _ptr(d_sc)
    gr.dL_drotations = _ptr(d_rot)
    if N > 0:
        with _Timed(timers, "backward"):
            native.check(lib.cfgs_plain_backward(C.byref(s), C.byref(g), state.radii.data_ptr(),
                                                 state.geom.data_ptr(), state.image.data_ptr(), state.work.data_ptr(),
                                                 state.capacity, grad_color.data_ptr(), _ptr(grad_depth),
                                                 _ptr(grad_alpha), C.byref(gr), st), "cfgs_plain_backward")
    return d_m2, d_col, d_op, d_m3, d_cov, d_sh, d_sc, d_rot
