"""The allocation-free backward (cfgs_backward_noalloc) against the allocating one.

cfgs_backward_noalloc exists for callers that cannot allocate device memory when they
call the backward (plugin hosts that hand over only input and output buffers, services
that must not allocate once serving). Its scratch is a fixed array inside libcfgs.so,
shared by every call and keeping the last call's contents. This test calls it through
the C ABI:
- first on an unrelated scene (other size, seed and instance count), so the array holds
  records that the target scene does not need;
- then twice in a row on the target scene, each result compared bit for bit with
  cfgs_backward given a freshly allocated scratch buffer (both run the same kernels in
  the same order, so the gradients are identical, not merely close);
- with a binning workspace whose capacity is above the instance count;
- and, without device work, the size checks: capacity == CFGS_NOALLOC_MAX_INSTANCES
  passes them, a negative capacity is an invalid argument, and one above the maximum is
  refused as too large.
The file is named to be collected last.
"""
from __future__ import annotations

import ctypes as C

import pytest
import torch

from helpers import l1_image_grad, settings_for

pytestmark = pytest.mark.gpu

MAX_INSTANCES = 655360  # CFGS_NOALLOC_MAX_INSTANCES in include/cfgs.h
INVALID_ARGUMENT, TOO_LARGE = 1, 5


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


class _Case:
    """One forward through the C ABI into workspaces whose binning capacity is
    `capacity_extra` instances above the scene's instance count, plus the upstream
    gradients of the backward."""

    def __init__(self, dgr, sc, capacity_extra=0):
        from cfgs import native, raster
        lib = native.load()
        dev = torch.device("cuda")
        self.rs = settings_for(dgr, sc)
        s = sc.to(dev)
        self.keep: list = []
        self.cs = raster.make_settings(self.rs, self.keep)
        self.cg = raster.make_gaussians(s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
        self.keep += [s]
        self.N, self.M = sc.n, int(sc.shs.shape[1])
        self.stream = torch.cuda.current_stream().cuda_stream
        W, H = sc.camera.width, sc.camera.height
        self.geom = torch.empty(lib.cfgs_geom_bytes(self.N), dtype=torch.uint8, device=dev)
        self.image = torch.empty(lib.cfgs_image_bytes(W, H), dtype=torch.uint8, device=dev)
        self.radii = torch.empty(self.N, dtype=torch.int32, device=dev)
        native.check(lib.cfgs_preprocess_forward(C.byref(self.cs), C.byref(self.cg), self.geom.data_ptr(),
                                                 self.image.data_ptr(), self.radii.data_ptr(), self.stream),
                     "cfgs_preprocess_forward")
        counts = native.Counts()
        native.check(lib.cfgs_read_counts(self.image.data_ptr(), C.byref(counts), self.stream), "cfgs_read_counts")
        self.K = int(counts.num_rendered)
        self.capacity = self.K + capacity_extra
        self.binning = torch.empty(lib.cfgs_binning_bytes(self.capacity), dtype=torch.uint8, device=dev)
        color = torch.empty(3, H, W, device=dev)
        depth = torch.empty(1, H, W, device=dev)
        alpha = torch.empty(1, H, W, device=dev)
        native.check(lib.cfgs_render_forward(C.byref(self.cs), C.byref(self.cg), self.geom.data_ptr(),
                                             self.image.data_ptr(), self.binning.data_ptr(), self.capacity,
                                             color.data_ptr(), depth.data_ptr(), alpha.data_ptr(), self.stream),
                     "cfgs_render_forward")
        self.g_color = l1_image_grad(color, s.target).contiguous()
        gen = torch.Generator().manual_seed(3)
        self.g_depth = (torch.randn(1, H, W, generator=gen) * 1e-3).to(dev)
        self.g_alpha = (torch.randn(1, H, W, generator=gen) * 1e-3).to(dev)

    def args(self, capacity=None):
        return (C.byref(self.cs), C.byref(self.cg), self.radii.data_ptr(), self.geom.data_ptr(),
                self.image.data_ptr(), self.binning.data_ptr(), self.capacity if capacity is None else capacity)

    def grads_in(self):
        return (self.g_color.data_ptr(), self.g_depth.data_ptr(), self.g_alpha.data_ptr())

    def allocating(self):
        from cfgs import native
        lib = native.load()
        scratch = torch.empty(lib.cfgs_backward_scratch_bytes(self.capacity), dtype=torch.uint8, device="cuda")
        bufs, gr = _grad_buffers(self.N, self.M, "cuda")
        rc = lib.cfgs_backward(*self.args(), scratch.data_ptr(), *self.grads_in(), C.byref(gr), self.stream)
        assert rc == 0
        torch.cuda.synchronize()
        return bufs

    def noalloc(self, fn):
        bufs, gr = _grad_buffers(self.N, self.M, "cuda")
        rc = fn(*self.args(), *self.grads_in(), C.byref(gr), self.stream)
        assert rc == 0, f"status {rc}"
        torch.cuda.synchronize()
        return bufs


def _assert_same(got, want, label):
    for name in want:
        assert torch.isfinite(got[name]).all(), f"{label}: {name} not fully written"
        assert torch.equal(got[name], want[name]), f"{label}: {name} differs from cfgs_backward"


def test_backward_noalloc_matches_cfgs_backward():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as dgr
    from cfgs import native, scenes
    noalloc = _bind(native.load())

    # an unrelated scene first: the shared array then holds records the target does not use
    other = _Case(dgr, scenes.scene_small(n=9000, width=200, height=150, seed=41))
    target = _Case(dgr, scenes.scene_small(n=16384, width=256, height=256, seed=0))
    assert 0 < other.K <= MAX_INSTANCES and 0 < target.K <= MAX_INSTANCES and other.K != target.K
    _assert_same(other.noalloc(noalloc), other.allocating(), "unrelated scene")

    want = target.allocating()
    for call in range(2):
        _assert_same(target.noalloc(noalloc), want, f"call {call}")

    # a binning workspace with room for more instances than the scene has
    roomy = _Case(dgr, scenes.scene_small(n=16384, width=256, height=256, seed=0), capacity_extra=5000)
    assert roomy.capacity > roomy.K
    want_roomy = roomy.allocating()
    _assert_same(roomy.noalloc(noalloc), want_roomy, "capacity above K")
    _assert_same(want_roomy, want, "capacity above K vs exact capacity")


def test_backward_noalloc_size_checks():
    """Host-side checks only: no kernel runs in any of these calls."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import native
    noalloc = _bind(native.load())
    g = native.Gaussians()
    g.num_gaussians = 1
    grads = native.Gradients()
    stream = torch.cuda.current_stream().cuda_stream
    # capacity == maximum passes the size check; the null settings are then rejected
    assert noalloc(None, C.byref(g), None, None, None, None, MAX_INSTANCES, None, None, None, C.byref(grads),
                   stream) == INVALID_ARGUMENT
    assert noalloc(None, C.byref(g), None, None, None, None, MAX_INSTANCES + 1, None, None, None, C.byref(grads),
                   stream) == TOO_LARGE
    assert noalloc(None, C.byref(g), None, None, None, None, -1, None, None, None, C.byref(grads),
                   stream) == INVALID_ARGUMENT
