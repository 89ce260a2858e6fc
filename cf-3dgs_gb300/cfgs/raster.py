"""Host side of the rasteriser: workspace allocation, the two forward phases, the
backward, and the autograd Function behind `diff_gaussian_rasterization`.

Everything here calls libcfgs.so through its C ABI; there is no other execution path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import autotune, native

_EMPTY = None


def _ptr(t: torch.Tensor | None) -> int | None:
    if t is None or t.numel() == 0:
        return None
    return t.data_ptr()


def _f32(t: torch.Tensor | None) -> torch.Tensor | None:
    if t is None or t.numel() == 0:
        return None
    if t.dtype != torch.float32:
        t = t.float()
    return t.contiguous()


def _req(t: torch.Tensor) -> torch.Tensor:
    if t.dtype != torch.float32:
        t = t.float()
    return t.contiguous()


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def make_settings(rs, keep: list, schedule=None) -> native.Settings:
    """Packs a GaussianRasterizationSettings into the C struct. Tensors are made
    contiguous float32 and appended to `keep` so they outlive the call. The render
    schedule is `schedule` (an autotune.Schedule) or the calling thread's current one."""
    bg = _f32(rs.bg)
    view = _f32(rs.viewmatrix)
    proj = _f32(rs.projmatrix)
    campos = _f32(rs.campos)
    keep.extend([bg, view, proj, campos])
    s = native.Settings()
    s.image_height = int(rs.image_height)
    s.image_width = int(rs.image_width)
    s.tanfovx = float(rs.tanfovx)
    s.tanfovy = float(rs.tanfovy)
    s.bg = _ptr(bg)
    s.scale_modifier = float(rs.scale_modifier)
    s.viewmatrix = _ptr(view)
    s.projmatrix = _ptr(proj)
    s.sh_degree = int(rs.sh_degree)
    s.campos = _ptr(campos)
    s.prefiltered = int(bool(rs.prefiltered))
    s.debug = int(bool(rs.debug))
    s.schedule = autotune.c_schedule() if schedule is None else autotune.c_schedule(schedule)
    return s


def make_gaussians(means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp) -> native.Gaussians:
    g = native.Gaussians()
    g.num_gaussians = int(means3D.shape[0])
    g.means3D = _ptr(means3D)
    g.opacities = _ptr(opacities)
    g.shs = _ptr(shs)
    g.sh_coeffs = int(shs.shape[1]) if shs is not None and shs.numel() else 0
    g.colors_precomp = _ptr(colors_precomp)
    g.scales = _ptr(scales)
    g.rotations = _ptr(rotations)
    g.cov3D_precomp = _ptr(cov3D_precomp)
    return g


@dataclass
class ForwardState:
    """Workspaces of one forward call (the upstream geom/binning/image buffers)."""
    geom: torch.Tensor
    image: torch.Tensor
    binning: torch.Tensor
    num_rendered: int
    radii: torch.Tensor


class _Timed:
    """Brackets one library call with CUDA events on the current stream when `timers`
    (a dict phase -> list of (start, stop) events) is given."""

    def __init__(self, timers, name):
        self.timers, self.name = timers, name

    def __enter__(self):
        if self.timers is not None:
            self.ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            self.ev[0].record()

    def __exit__(self, *exc):
        if self.timers is not None:
            self.ev[1].record()
            self.timers.setdefault(self.name, []).append(self.ev)


_SIDE_STREAMS: dict = {}


def _read_counts_after(image: torch.Tensor, ready: torch.cuda.Event, dev) -> native.Counts:
    """The CfgsCounts at the head of an image workspace, copied to pinned host memory
    on a side stream once `ready` has completed (work enqueued after it on the current
    stream keeps running). Waits for that copy only."""
    side = _SIDE_STREAMS.get(dev)
    if side is None:
        side = _SIDE_STREAMS[dev] = torch.cuda.Stream(dev)
    host = torch.empty(C.sizeof(native.Counts), dtype=torch.uint8, pin_memory=True)
    with torch.cuda.stream(side):
        side.wait_event(ready)
        host.copy_(image[: host.numel()], non_blocking=True)
        done = torch.cuda.Event()
        done.record(side)
    image.record_stream(side)
    done.synchronize()
    return native.Counts.from_buffer_copy(host.numpy().tobytes())


def forward(rs, means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp, timers=None):
    """Runs both forward phases. Returns (color, radii, depth, alpha, ForwardState)."""
    lib = native.load()
    dev = means3D.device
    if dev.type != "cuda":
        raise RuntimeError("diff_gaussian_rasterization (GB300) needs CUDA tensors; got " + str(dev))
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
    # K is final here; the depth sort does not need it, so it is enqueued before the host
    # waits for K (read on a side stream), and keeps the GPU busy meanwhile.
    k_ready = torch.cuda.Event()
    k_ready.record(torch.cuda.current_stream(dev))
    with _Timed(timers, "depth_sort"):
        native.check(lib.cfgs_depth_order(N, geom.data_ptr(), st), "cfgs_depth_order")
    counts = _read_counts_after(image, k_ready, dev)
    if counts.flags & native.FLAG_FRUSTUM_VIOLATION:
        raise RuntimeError("prefiltered=True but a Gaussian lies at view z <= 0.2 (outside the frustum)")
    if counts.flags & native.FLAG_CAPACITY_OVERFLOW:
        raise RuntimeError("more than 2^31 tile instances")
    K = int(counts.num_rendered)
    binning = torch.empty(lib.cfgs_binning_bytes(K), dtype=torch.uint8, device=dev)
    color = torch.empty((3, H, W), dtype=torch.float32, device=dev)
    depth = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    alpha = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    with _Timed(timers, "bin"):
        native.check(lib.cfgs_bin_instances(C.byref(s), C.byref(g), geom.data_ptr(), image.data_ptr(),
                                            binning.data_ptr(), K, st), "cfgs_bin_instances")
    with _Timed(timers, "composite"):
        native.check(lib.cfgs_composite_forward(C.byref(s), N, geom.data_ptr(), image.data_ptr(), binning.data_ptr(),
                                                K, color.data_ptr(), depth.data_ptr(), alpha.data_ptr(), st),
                     "cfgs_composite_forward")
    return color, radii, depth, alpha, ForwardState(geom, image, binning, K, radii)


def backward(rs, state: ForwardState, means3D, opacities, shs, colors_precomp, scales, rotations,
             cov3D_precomp, grad_color, grad_depth, grad_alpha, timers=None):
    """Returns (dmeans2D, dcolors, dopacity, dmeans3D, dcov3D, dsh, dscales, drotations)."""
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
    K = state.num_rendered
    scratch = torch.empty(lib.cfgs_backward_scratch_bytes(K), dtype=torch.uint8, device=dev)
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
        with _Timed(timers, "render_bwd"):
            native.check(lib.cfgs_render_backward(C.byref(s), N, state.geom.data_ptr(), state.image.data_ptr(),
                                                  state.binning.data_ptr(), K, scratch.data_ptr(),
                                                  grad_color.data_ptr(), _ptr(grad_depth), _ptr(grad_alpha), st),
                         "cfgs_render_backward")
        with _Timed(timers, "preprocess_bwd"):
            native.check(lib.cfgs_preprocess_backward(C.byref(s), C.byref(g), state.radii.data_ptr(),
                                                      state.geom.data_ptr(), state.image.data_ptr(), K,
                                                      scratch.data_ptr(), C.byref(gr), st),
                         "cfgs_preprocess_backward")
    return d_m2, d_col, d_op, d_m3, d_cov, d_sh, d_sc, d_rot


def _none_if_empty(t):
    return None if t is None or t.numel() == 0 else t


class RasterizeGaussiansFn(torch.autograd.Function):
    """autograd Function of rasterize_gaussians: outputs (color, radii, depth, alpha);
    gradients flow to means3D, means2D (screen-space NDC), sh or colors_precomp,
    opacities, scales and rotations or cov3Ds_precomp."""

    @staticmethod
    def forward(ctx, means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                raster_settings):
        sh = _f32(_none_if_empty(sh))
        colors_precomp = _f32(_none_if_empty(colors_precomp))
        scales = _f32(_none_if_empty(scales))
        rotations = _f32(_none_if_empty(rotations))
        cov3Ds_precomp = _f32(_none_if_empty(cov3Ds_precomp))
        means3D_c = _req(means3D)
        opac = _req(opacities)
        args = (means3D_c, opac, sh, colors_precomp, scales, rotations, cov3Ds_precomp)
        try:
            color, radii, depth, alpha, state = forward(raster_settings, *args)
        except Exception:
            if raster_settings.debug:
                torch.save((raster_settings, args), "snapshot_fw.dump")
                print("\nAn error occurred in the rasteriser forward; inputs saved to snapshot_fw.dump.")
            raise
        ctx.raster_settings = raster_settings
        ctx.state = state
        ctx.has = (sh is not None, colors_precomp is not None, cov3Ds_precomp is not None)
        ctx.save_for_backward(*[a if a is not None else torch.empty(0) for a in args])
        ctx.mark_non_differentiable(radii)
        # Outputs the loss does not use (often depth and alpha) arrive as None rather than
        # as zero tensors, so the backward skips their terms (the gradients are the same).
        ctx.set_materialize_grads(False)
        return color, radii, depth, alpha

    @staticmethod
    def backward(ctx, grad_color, grad_radii, grad_depth, grad_alpha):
        means3D, opac, sh, colors_precomp, scales, rotations, cov3Ds = ctx.saved_tensors
        has_sh, has_col, has_cov = ctx.has
        sh = sh if has_sh else None
        colors_precomp = colors_precomp if has_col else None
        cov3Ds = cov3Ds if has_cov else None
        if not has_cov:
            pass
        else:
            scales = rotations = None
        rs = ctx.raster_settings
        if grad_color is None:
            grad_color = torch.zeros((3, int(rs.image_height), int(rs.image_width)), dtype=torch.float32,
                                     device=means3D.device)
        try:
            d_m2, d_col, d_op, d_m3, d_cov, d_sh, d_sc, d_rot = backward(
                rs, ctx.state, means3D, opac, sh, colors_precomp, scales, rotations, cov3Ds,
                grad_color, grad_depth, grad_alpha)
        except Exception:
            if rs.debug:
                torch.save((rs,), "snapshot_bw.dump")
                print("\nAn error occurred in the rasteriser backward; settings saved to snapshot_bw.dump.")
            raise
        return (d_m3, d_m2, d_sh if has_sh else None, d_col if has_col else None, d_op,
                d_sc, d_rot, d_cov if has_cov else None, None)


def mark_visible(positions: torch.Tensor, viewmatrix: torch.Tensor, projmatrix: torch.Tensor) -> torch.Tensor:
    lib = native.load()
    pos = _req(positions)
    view = _f32(viewmatrix)
    proj = _f32(projmatrix)
    n = int(positions.shape[0])
    vis = torch.empty(n, dtype=torch.uint8, device=positions.device)
    native.check(lib.cfgs_mark_visible(n, _ptr(pos), _ptr(view), _ptr(proj), vis.data_ptr() if n else None,
                                       stream_handle(positions.device)), "cfgs_mark_visible")
    return vis.bool()


def kernel_launches(width: int, height: int) -> dict:
    """Kernels the forward and backward launch for one image (N > 0): preprocess and
    the K sum; binning = depth sort (4 radix passes of count/scan/scatter), rank sums,
    emission, tile sort (count/scan/scatter per pass of at most 8 tile-index bits) and
    tile ranges; compositing; render backward; preprocess backward. (Memory clears the
    library enqueues with cudaMemsetAsync are not counted.)"""
    tiles = ((width + 15) // 16) * ((height + 15) // 16)
    bits = 1
    while bits < 31 and (1 << bits) < tiles:
        bits += 1
    tile_passes = (bits + 7) // 8
    out = {"preprocess": 2, "bin": 4 * 3 + 2 + 3 * tile_passes + 1, "composite": 1, "render_bwd": 1,
           "preprocess_bwd": 1}
    out["total"] = sum(out.values())
    return out


def inspect_state(state: ForwardState, width: int, height: int) -> dict:
    """Typed views of the forward workspaces (for tests and debugging)."""
    import torch as _t
    N = int(state.radii.shape[0])
    K = state.num_rendered
    gl = native.geom_layout(N)
    il = native.image_layout(width, height)
    bl = native.binning_layout(K)
    T = ((width + 15) // 16) * ((height + 15) // 16)
    HW = width * height

    def view(buf, off, count, dtype, elem):
        return buf[off: off + count * elem].view(dtype)

    g, im, b = state.geom, state.image, state.binning
    out = {
        "xy": view(g, gl["xy"], 2 * N, _t.float32, 4).reshape(N, 2),
        "conic_op": view(g, gl["conic_op"], 4 * N, _t.float32, 4).reshape(N, 4),
        "rgbd": view(g, gl["rgbd"], 4 * N, _t.float32, 4).reshape(N, 4),
        "rect": view(g, gl["rect"], 2 * N, _t.int32, 4).reshape(N, 2),
        "touched": view(g, gl["touched"], N, _t.int32, 4),
        "offset": view(g, gl["offset"], N, _t.int32, 4),
        "clamped": view(g, gl["clamped"], N, _t.uint8, 1),
        "counts": view(im, il["counts"], 2, _t.int32, 4),
        "tile_range": view(im, il["tile_range"], T + 1, _t.int32, 4),
        "final_T": view(im, il["final_T"], HW, _t.float32, 4),
        "n_contrib": view(im, il["n_contrib"], HW, _t.int32, 4),
        "sorted_gid": view(b, bl["sorted_gid"], K, _t.int32, 4),
        "sorted_pidx": view(b, bl["sorted_pidx"], K, _t.int32, 4),
    }
    return out
