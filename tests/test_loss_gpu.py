"""Fused L1 loss (cfgs_l1_loss_forward / cfgs_l1_loss_backward) against PyTorch fp32
autograd of utils/loss_utils.py's l1_loss (torch.abs(x - gt).mean()), with and without
the clamp the pose solve applies first. The gradient is bit-identical (the same sign
times g / n, the same clamp mask); the mean agrees to 1e-6 relative (a different
summation order: fixed blocks and a float64 fold here)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def loss_mod():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cfgs import loss
    return loss


def _inputs(shape, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.2, 1.2, shape).astype(np.float32)   # both sides of the clamp
    t = rng.uniform(0, 1, shape).astype(np.float32)
    flat_x, flat_t = x.reshape(-1), t.reshape(-1)
    k = min(8, flat_x.size)
    flat_t[:k // 2] = flat_x[:k // 2]                      # c - t = 0: sign 0
    flat_x[k // 2:k] = np.array([0.0, 1.0, -0.0, 1.0], np.float32)[: k - k // 2]  # clamp boundaries
    return x, t


def _torch_ref(x, t, clamp, g=1.0):
    xr = torch.tensor(x, device=DEV, requires_grad=True)
    tt = torch.tensor(t, device=DEV)
    c = xr.clamp(0, 1) if clamp else xr
    v = torch.abs(c - tt).mean()
    (v * g if g != 1.0 else v).backward()
    return v.detach(), xr.grad


@pytest.mark.parametrize("clamp", [False, True])
@pytest.mark.parametrize("shape", [(3, 1080, 1920), (3, 37, 53), (1,), (5,), (4099,), (2, 3, 21, 19)])
def test_l1_matches_torch(loss_mod, shape, clamp):
    x, t = _inputs(shape, seed=sum(shape) + clamp)
    ref_v, ref_g = _torch_ref(x, t, clamp)
    xx = torch.tensor(x, device=DEV, requires_grad=True)
    v = loss_mod.l1_loss(xx, torch.tensor(t, device=DEV), clamp=clamp)
    v.backward()
    assert abs(float(v.detach()) - float(ref_v)) <= 1e-6 * abs(float(ref_v)) + 1e-12
    assert torch.equal(xx.grad, ref_g)
    # one-pass form: same loss bits as the autograd forward, same gradient as autograd
    v1, g1 = loss_mod.l1_loss_and_grad(torch.tensor(x, device=DEV), torch.tensor(t, device=DEV), clamp=clamp)
    assert float(v1) == float(v.detach())
    assert torch.equal(g1, ref_g)


def test_l1_upstream_gradient_and_misaligned_views(loss_mod):
    x, t = _inputs((10_001,), seed=5)
    ref_v, ref_g = _torch_ref(x[1:], t[1:], True, g=0.37)
    xb = torch.tensor(x, device=DEV)
    tb = torch.tensor(t, device=DEV)
    xv = xb[1:].requires_grad_(True)                      # 4-byte offset: the scalar path
    v = loss_mod.l1_loss(xv, tb[1:], clamp=True)
    (v * 0.37).backward()
    assert abs(float(v.detach()) - float(ref_v)) <= 1e-6 * abs(float(ref_v))
    torch.testing.assert_close(xv.grad, ref_g, rtol=2.5e-7, atol=0.0)  # within one rounding of g / n


def test_l1_empty_is_nan_and_deterministic(loss_mod):
    e = torch.empty(0, device=DEV)
    assert torch.isnan(loss_mod.l1_loss(e, e))
    x, t = _inputs((3, 360, 640), seed=9)
    xt, tt = torch.tensor(x, device=DEV), torch.tensor(t, device=DEV)
    a = [float(loss_mod.l1_loss(xt, tt, clamp=True)) for _ in range(3)]
    assert a[0] == a[1] == a[2]

