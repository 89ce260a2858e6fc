"""Gaussian-parameter optimisation on the GPU: the fused Adam against torch.optim.Adam
(bit for bit) and densify_and_prune against the reference's functions restated in
PyTorch (oracle/densify_oracle.py) on the same split draws: identical counts and row
order, copied rows bit for bit, split children within float32 rounding (1e-6)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def dz():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cfgs import densify
    return densify


def _model(n, seed):
    g = torch.Generator().manual_seed(seed)
    return {"xyz": torch.randn(n, 3, generator=g), "f_dc": torch.randn(n, 1, 3, generator=g),
            "f_rest": 0.1 * torch.randn(n, 15, 3, generator=g), "opacity": 2.0 * torch.randn(n, 1, generator=g),
            "scaling": torch.randn(n, 3, generator=g) - 4.0, "rotation": torch.randn(n, 4, generator=g)}


LRS = {"xyz": 1.6e-4 * 3.2, "f_dc": 2.5e-3, "f_rest": 2.5e-3 / 20, "opacity": 0.05, "scaling": 5e-3,
       "rotation": 1e-3}


def test_gaussian_adam_matches_torch(dz):
    p0 = _model(3000, 0)
    opt = dz.GaussianOptimizer({k: v.to(DEV) for k, v in p0.items()}, LRS)
    ref = {k: torch.nn.Parameter(v.clone().to(DEV)) for k, v in p0.items()}
    topt = torch.optim.Adam([{"params": [ref[k]], "lr": LRS[k], "name": k} for k in dz.GROUPS], lr=0.0, eps=1e-15)
    g = torch.Generator().manual_seed(7)
    for _ in range(4):
        grads = {k: torch.randn(v.shape, generator=g).to(DEV) * 0.01 for k, v in p0.items()}
        opt.step(grads)
        for k in dz.GROUPS:
            ref[k].grad = grads[k].clone()
        topt.step()
    for k in dz.GROUPS:
        np.testing.assert_array_equal(opt.params[k].cpu().numpy(), ref[k].detach().cpu().numpy(), err_msg=k)
        st = topt.state[ref[k]]
        np.testing.assert_array_equal(opt.exp_avg[k].cpu().numpy(), st["exp_avg"].cpu().numpy(), err_msg=k)
        np.testing.assert_array_equal(opt.exp_avg_sq[k].cpu().numpy(), st["exp_avg_sq"].cpu().numpy(), err_msg=k)


def test_densification_stats(dz):
    n = 5000
    opt = dz.GaussianOptimizer({k: v.to(DEV) for k, v in _model(n, 1).items()}, LRS)
    g = torch.Generator().manual_seed(2)
    acc, den = torch.zeros(n), torch.zeros(n)
    for _ in range(3):
        grad2d = torch.randn(n, 3, generator=g)
        radii = (torch.rand(n, generator=g) > 0.3).int() * 5
        opt.add_densification_stats(grad2d.to(DEV), radii.to(DEV))
        vis = radii > 0
        acc[vis] += torch.norm(grad2d[vis, :2], dim=-1)
        den[vis] += 1
    np.testing.assert_allclose(opt.grad_accum.cpu().numpy(), acc.numpy(), rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(opt.denom.cpu().numpy(), den.numpy())


@pytest.mark.parametrize("max_screen_size", [20, None])
def test_densify_and_prune_matches_reference(dz, max_screen_size):
    from oracle import densify_oracle
    n = 20000
    p0 = _model(n, 3)
    g = torch.Generator().manual_seed(4)
    # gradients well away from the threshold; a third of the points never seen (nan -> 0)
    accum = torch.where(torch.rand(n, generator=g) < 0.5, torch.full((n,), 5e-4), torch.full((n,), 1e-5))
    denom = torch.where(torch.rand(n, generator=g) < 0.66, torch.ones(n), torch.zeros(n))
    accum = accum * denom
    # scalings away from the clone/split boundary (percent_dense * extent = 0.03)
    s = p0["scaling"]
    s[s.exp().max(1).values.sub(0.03).abs() < 1e-3] -= 0.5
    p0["opacity"][torch.sigmoid(p0["opacity"]).sub(0.005).abs() < 1e-4] += 1.0
    opt = dz.GaussianOptimizer({k: v.to(DEV) for k, v in p0.items()}, LRS)
    for k in dz.GROUPS:  # non-trivial moments to follow through the reshuffle
        opt.exp_avg[k].copy_(torch.randn(opt.exp_avg[k].shape, generator=g).to(DEV))
        opt.exp_avg_sq[k].copy_(torch.rand(opt.exp_avg_sq[k].shape, generator=g).to(DEV))
    m0 = {k: v.cpu().clone() for k, v in opt.exp_avg.items()}
    v0 = {k: v.cpu().clone() for k, v in opt.exp_avg_sq.items()}
    opt.grad_accum.copy_(accum.to(DEV))
    opt.denom.copy_(denom.to(DEV))
    kw = dict(max_grad=2e-4, min_opacity=0.005, extent=3.0, max_screen_size=max_screen_size, percent_dense=0.01)
    # split count from the plan, then the same draws for both sides
    splits = int(((accum / denom).nan_to_num(0.0) >= 2e-4).logical_and(p0["scaling"].exp().max(1).values > 0.03).sum())
    z = torch.randn(2, splits, 3, generator=g)
    res = opt.densify_and_prune(z=z.to(DEV), **kw)
    P, M, V = densify_oracle.densify_and_prune(p0, m0, v0, accum, denom, z=z, **kw)
    assert res["total"] == P["xyz"].shape[0] and res["split"] == splits
    assert res["cloned"] > 0 and res["children_per_copy"] > 0 and res["kept"] < n
    n_copy = res["kept"] + res["cloned"]
    for k in dz.GROUPS:
        got = opt.params[k].cpu()
        if k in ("xyz", "scaling"):
            np.testing.assert_array_equal(got[:n_copy].numpy(), P[k][:n_copy].numpy(), err_msg=k)
            np.testing.assert_allclose(got[n_copy:].numpy(), P[k][n_copy:].numpy(), rtol=0, atol=1e-6, err_msg=k)
        else:
            np.testing.assert_array_equal(got.numpy(), P[k].numpy(), err_msg=k)
        np.testing.assert_array_equal(opt.exp_avg[k].cpu().numpy(), M[k].numpy(), err_msg=k)
        np.testing.assert_array_equal(opt.exp_avg_sq[k].cpu().numpy(), V[k].numpy(), err_msg=k)
    assert float(opt.grad_accum.abs().sum()) == 0.0 and opt.denom.shape[0] == res["total"]
