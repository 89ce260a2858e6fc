"""L1 photometric loss on the GPU: the `l1_loss` of utils/loss_utils.py:15-16 (and of
trainer/losses.py:139-140), mean |x - gt| over every element, optionally of
clamp(x, 0, 1) as the pose solve forms it (scene/gaussian_model_cf.py:885 clamps the
render, trainer/losses.py:98-136 takes the L1 of it). One kernel pass per direction
through cfgs_l1_loss_forward / cfgs_l1_loss_backward; the gradient is autograd's
(sign times g / n, zero where the clamp cuts)."""
from __future__ import annotations

import torch

from . import native
from .raster import _ptr, stream_handle


def _operands(x: torch.Tensor, gt: torch.Tensor):
    if not x.is_cuda or gt.device != x.device:
        raise ValueError("l1_loss: both tensors must be CUDA tensors on one device")
    if x.shape != gt.shape:
        raise ValueError(f"l1_loss: shapes differ: {tuple(x.shape)} vs {tuple(gt.shape)}")
    return x.detach().float().contiguous(), gt.detach().float().contiguous()


class L1LossFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, gt: torch.Tensor, clamp: bool) -> torch.Tensor:
        a, b = _operands(x, gt)
        lib = native.load()
        n = a.numel()
        scratch = torch.empty(int(lib.cfgs_l1_loss_scratch_bytes(n)), dtype=torch.uint8, device=a.device)
        out = torch.empty((), dtype=torch.float32, device=a.device)
        native.check(lib.cfgs_l1_loss_forward(n, _ptr(a), _ptr(b), int(clamp), scratch.data_ptr(), out.data_ptr(),
                                              None, stream_handle(a.device)), "cfgs_l1_loss_forward")
        ctx.save_for_backward(a, b)
        ctx.clamp, ctx.in_shape, ctx.in_dtype = bool(clamp), x.shape, x.dtype
        return out

    @staticmethod
    def backward(ctx, grad: torch.Tensor):
        a, b = ctx.saved_tensors
        lib = native.load()
        g = grad.detach().float().reshape(()).contiguous()
        dx = torch.empty_like(a)
        native.check(lib.cfgs_l1_loss_backward(a.numel(), _ptr(a), _ptr(b), int(ctx.clamp), g.data_ptr(), _ptr(dx),
                                               stream_handle(a.device)), "cfgs_l1_loss_backward")
        return dx.reshape(ctx.in_shape).to(ctx.in_dtype), None, None


def l1_loss(network_output: torch.Tensor, gt: torch.Tensor, clamp: bool = False) -> torch.Tensor:
    """mean |network_output - gt| (utils/loss_utils.py:15); with clamp=True the mean of
    |clamp(network_output, 0, 1) - gt|. Gradients flow to network_output only."""
    if gt.requires_grad:
        raise NotImplementedError("l1_loss: gradients flow to network_output only (gt is the target)")
    return L1LossFn.apply(network_output, gt, clamp)


def l1_loss_and_grad(x: torch.Tensor, gt: torch.Tensor, clamp: bool = False,
                     out: torch.Tensor | None = None, grad_out: torch.Tensor | None = None,
                     scratch: torch.Tensor | None = None):
    """The loss and its gradient (upstream gradient 1) in one pass, outside autograd:
    for a loss that ends the graph (a training or pose-solve step that calls the
    rasteriser's backward itself). Returns (loss [], dL/dx shaped like x). The optional
    buffers make the call allocation-free."""
    a, b = _operands(x, gt)
    lib = native.load()
    n = a.numel()
    if scratch is None:
        scratch = torch.empty(int(lib.cfgs_l1_loss_scratch_bytes(n)), dtype=torch.uint8, device=a.device)
    if out is None:
        out = torch.empty((), dtype=torch.float32, device=a.device)
    if grad_out is None:
        grad_out = torch.empty_like(a)
    native.check(lib.cfgs_l1_loss_forward(n, _ptr(a), _ptr(b), int(clamp), scratch.data_ptr(), out.data_ptr(),
                                          _ptr(grad_out), stream_handle(a.device)), "cfgs_l1_loss_forward")
    return out, grad_out.view(x.shape)
