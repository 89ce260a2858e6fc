"""Fused SSIM (cfgs_ssim_forward / cfgs_ssim_backward) against the float64 oracle of
utils/loss_utils.py's ssim (itself pinned to the reference's code by
tests/test_golden_cpu.py). Tolerances: mean SSIM 1e-5 absolute, d SSIM / d img1 1e-4
relative (with the floor of helpers.grad_close)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import assert_grad_close

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def ssim_mod():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cfgs import ssim
    return ssim


def _pair(shape, seed, noise=0.1):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0, 1, shape).astype(np.float32)
    b = np.clip(a + rng.normal(0, noise, shape), 0, 1).astype(np.float32)
    return a, b


@pytest.mark.parametrize("shape", [(3, 64, 96), (3, 37, 53), (1, 5, 7), (3, 360, 640), (2, 3, 21, 19)])
def test_ssim_matches_oracle(ssim_mod, shape):
    from oracle import ssim_oracle
    a, b = _pair(shape, seed=sum(shape))
    x = torch.tensor(a, device=DEV, requires_grad=True)
    y = torch.tensor(b, device=DEV)
    v = ssim_mod.ssim(x, y)
    v.backward()
    chw = (-1,) + shape[-2:]
    ref_v, ref_g = ssim_oracle.ssim(a.reshape(chw), b.reshape(chw), with_grad=True)
    assert abs(float(v.detach()) - ref_v) <= 1e-5
    assert_grad_close("dssim/dimg1", x.grad.cpu().numpy().reshape(chw), ref_g)


def test_ssim_loss_scaling_and_identity(ssim_mod):
    """The CF-3DGS weighting 0.2 (1 - SSIM) scales the gradient; SSIM(x, x) = 1."""
    from oracle import ssim_oracle
    a, b = _pair((3, 48, 80), seed=5, noise=0.2)
    x = torch.tensor(a, device=DEV, requires_grad=True)
    loss = 0.2 * (1.0 - ssim_mod.ssim(x, torch.tensor(b, device=DEV)))
    loss.backward()
    _, ref_g = ssim_oracle.ssim(a, b, with_grad=True)
    assert_grad_close("d loss/dimg1", x.grad.cpu().numpy(), -0.2 * ref_g)
    same = ssim_mod.ssim(torch.tensor(a, device=DEV), torch.tensor(a, device=DEV))
    assert abs(float(same) - 1.0) < 1e-5


def test_ssim_deterministic(ssim_mod):
    a, b = _pair((3, 90, 120), seed=9)
    outs = []
    for _ in range(2):
        x = torch.tensor(a, device=DEV, requires_grad=True)
        v = ssim_mod.ssim(x, torch.tensor(b, device=DEV))
        v.backward()
        outs.append((float(v), x.grad.cpu().numpy().copy()))
    assert outs[0][0] == outs[1][0]
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_ssim_rejects_unsupported(ssim_mod):
    x = torch.rand(3, 8, 8, device=DEV)
    with pytest.raises(NotImplementedError):
        ssim_mod.ssim(x, x, window_size=7)
    with pytest.raises(NotImplementedError):
        ssim_mod.ssim(x, x.clone().requires_grad_(True))


def test_ssim_plain_staging_matches_oracle(ssim_mod):
    """A width that is not a multiple of four floats cannot be described by a tensor map;
    the kernels stage those tiles with plain loads (same results)."""
    from oracle import ssim_oracle
    a, b = _pair((3, 50, 83), seed=11)
    x = torch.tensor(a, device=DEV, requires_grad=True)
    v = ssim_mod.ssim(x, torch.tensor(b, device=DEV))
    v.backward()
    ref_v, ref_g = ssim_oracle.ssim(a, b, with_grad=True)
    assert abs(float(v.detach()) - ref_v) <= 1e-5
    assert_grad_close("dssim/dimg1", x.grad.cpu().numpy(), ref_g)
