"""SSIM loss on the GPU: the `ssim` of utils/loss_utils.py:33-38 (and the `_ssim` of
trainer/losses.py:147-196 without a mask), 11x11 Gaussian window, mean over every
channel and pixel, behind a torch.autograd.Function that calls cfgs_ssim_forward /
cfgs_ssim_backward. Gradients flow to img1 only (img2 is the target image)."""
from __future__ import annotations

import torch

from . import native
from .raster import _ptr, stream_handle


def _as_chw(img: torch.Tensor) -> torch.Tensor:
    if img.dim() == 3:
        return img
    if img.dim() == 4:
        return img.reshape(-1, img.shape[-2], img.shape[-1])  # batch x channel windows are independent
    raise ValueError("ssim expects [C,H,W] or [N,C,H,W] images")


class SsimFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, img1: torch.Tensor, img2: torch.Tensor) -> torch.Tensor:
        if not img1.is_cuda or img2.device != img1.device:
            raise ValueError("ssim: both images must be CUDA tensors on one device")
        a = _as_chw(img1).float().contiguous()
        b = _as_chw(img2).float().contiguous()
        if a.shape != b.shape:
            raise ValueError(f"ssim: shapes differ: {tuple(img1.shape)} vs {tuple(img2.shape)}")
        lib = native.load()
        C, H, W = (int(x) for x in a.shape)
        scratch = torch.empty(int(lib.cfgs_ssim_scratch_bytes(C, H, W)), dtype=torch.uint8, device=a.device)
        out = torch.empty((), dtype=torch.float32, device=a.device)
        native.check(lib.cfgs_ssim_forward(C, H, W, _ptr(a), _ptr(b), _ptr(scratch), out.data_ptr(),
                                           stream_handle(a.device)), "cfgs_ssim_forward")
        ctx.save_for_backward(a, b, scratch)
        ctx.in_shape, ctx.in_dtype = img1.shape, img1.dtype
        return out

    @staticmethod
    def backward(ctx, grad: torch.Tensor):
        a, b, scratch = ctx.saved_tensors
        lib = native.load()
        C, H, W = (int(x) for x in a.shape)
        g = grad.detach().float().reshape(()).contiguous()
        d1 = torch.empty_like(a)
        native.check(lib.cfgs_ssim_backward(C, H, W, _ptr(a), _ptr(b), _ptr(scratch), g.data_ptr(), _ptr(d1),
                                            stream_handle(a.device)), "cfgs_ssim_backward")
        return d1.reshape(ctx.in_shape).to(ctx.in_dtype), None


def ssim(img1: torch.Tensor, img2: torch.Tensor, window_size: int = 11, size_average: bool = True) -> torch.Tensor:
    """Mean SSIM of img1 against img2 (utils/loss_utils.py:33). Only the configuration
    CF-3DGS uses is built: an 11x11 window averaged over everything."""
    if window_size != 11 or not size_average:
        raise NotImplementedError("ssim: only window_size=11, size_average=True is implemented")
    if img2.requires_grad:
        raise NotImplementedError("ssim: gradients flow to img1 only (img2 is the target)")
    return SsimFn.apply(img1, img2)
