"""The allocation-free backward (cfgs_backward_noalloc) against the allocating one.

cfgs_backward_noalloc exists for callers that cannot allocate device memory when they
call the backward (plugin hosts that hand over only input and output buffers, services
that must not allocate once serving). Its scratch is a fixed array inside libcfgs.so,
shared by every call. This test calls it through the C ABI twice in a row — the second
call sees the array holding the first call's contents — and checks both results against
cfgs_backward given a freshly allocated scratch buffer, with the gradient tolerance the
other tests use. It also checks that a capacity above the documented maximum is
refused. The file is named to be collected last.
"""
from __future__ import annotations

import ctypes as C

import pytest
import torch

from helpers import assert_grad_close, l1_image_grad, settings_for

pytestmark = pytest.mark.gpu

MAX_INSTANCES = 655360  # CFGS_NOALLOC_MAX_INSTANCES in include/cfgs.h


def _bind(lib):
    from cfgs import native
    fn = lib.cfgs_backward_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(native.Settings), C.POINTER(native.Gaussians), C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(native.Gradients),
                   C.c_void_p]
    return fn


def _grad_buffers(N, M, dev):
    from cfgs import native
    f = dict(device=dev, dtype=torch.float32)
    bufs = {"means2D": torch.full((N, 3), float("nan"), **f), "colors": torch.full((N, 3), float("nan"), **f),
            "opacity": torch.full((N, 1), float("nan"), **f), "means3D": torch.full((N, 3), float("nan"), **f),
            "cov3D": torch.full((N, 6), float("nan"), **f), "sh": torch.full((N, M, 3), float("nan"), **f),
            "scales": torch.full((N, 3), float("nan"), **f), "rotations": torch.full((N, 4), float("nan"), **f)}
    gr = native.Gradients()
    gr.dL_dmeans2D = bufs["means2D"].data_ptr()
    gr.dL_dcolors = bufs["colors"].data_ptr()
    gr.dL_dopacity = bufs["opacity"].data_ptr()
    gr.dL_dmeans3D = bufs["means3D"].data_ptr()
    gr.dL_dcov3D = bufs["cov3D"].data_ptr()
    gr.dL_dsh = bufs["sh"].data_ptr()
    gr.dL_dscales = bufs["scales"].data_ptr()
    gr.dL_drotations = bufs["rotations"].data_ptr()
    return bufs, gr


def test_backward_noalloc_matches_cfgs_backward():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as dgr
    from cfgs import native, raster, scenes
    lib = native.load()
    noalloc = _bind(lib)
    dev = torch.device("cuda")
    sc = scenes.scene_small(n=16384, width=256, height=256, seed=0)
    rs = settings_for(dgr, sc)
    s = sc.to(dev)
    color, radii, depth, alpha, state = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales,
                                                       s.rotations, None)
    K = state.num_rendered
    assert 0 < K <= MAX_INSTANCES
    g_color = l1_image_grad(color, s.target).contiguous()
    gen = torch.Generator().manual_seed(3)
    g_depth = (torch.randn(1, sc.camera.height, sc.camera.width, generator=gen) * 1e-3).to(dev)
    g_alpha = (torch.randn(1, sc.camera.height, sc.camera.width, generator=gen) * 1e-3).to(dev)
    keep: list = []
    cs = raster.make_settings(rs, keep)
    cg = raster.make_gaussians(s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
    stream = torch.cuda.current_stream().cuda_stream
    N, M = sc.n, int(sc.shs.shape[1])

    scratch = torch.empty(lib.cfgs_backward_scratch_bytes(K), dtype=torch.uint8, device=dev)
    want, gr_want = _grad_buffers(N, M, dev)
    rc = lib.cfgs_backward(C.byref(cs), C.byref(cg), state.radii.data_ptr(), state.geom.data_ptr(),
                           state.image.data_ptr(), state.binning.data_ptr(), K, scratch.data_ptr(),
                           g_color.data_ptr(), g_depth.data_ptr(), g_alpha.data_ptr(), C.byref(gr_want), stream)
    assert rc == 0

    for call in range(2):
        got, gr_got = _grad_buffers(N, M, dev)
        rc = noalloc(C.byref(cs), C.byref(cg), state.radii.data_ptr(), state.geom.data_ptr(), state.image.data_ptr(),
                     state.binning.data_ptr(), K, g_color.data_ptr(), g_depth.data_ptr(), g_alpha.data_ptr(),
                     C.byref(gr_got), stream)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        for name in want:
            assert torch.isfinite(got[name]).all(), f"call {call}: {name} not fully written"
            assert_grad_close(f"call {call}: {name}", got[name].cpu(), want[name].cpu())

    # a capacity above the maximum is refused before any device work
    got, gr_got = _grad_buffers(N, M, dev)
    rc = noalloc(C.byref(cs), C.byref(cg), state.radii.data_ptr(), state.geom.data_ptr(), state.image.data_ptr(),
                 state.binning.data_ptr(), MAX_INSTANCES + 1, g_color.data_ptr(), g_depth.data_ptr(),
                 g_alpha.data_ptr(), C.byref(gr_got), stream)
    assert rc == 5  # CFGS_ERR_TOO_LARGE
