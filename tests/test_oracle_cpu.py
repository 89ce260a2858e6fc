"""CPU checks of the oracle itself: the C oracle (the bit-level checker of the GPU)
against the independent float64 autograd restatement, and the oracle's exp."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from helpers import assert_grad_close


def _both(sc, gseed=0, use_colors=False, use_cov=False):
    from oracle import torch_oracle as TO
    from oracle.c_oracle import Oracle
    cam = sc.camera
    g = torch.Generator().manual_seed(gseed)
    colors = torch.rand(sc.n, 3, generator=g) if use_colors else None
    cov = TO.cov3d(sc.scales.double(), sc.rotations.double(), 1.0).float() if use_cov else None
    o = Oracle.from_scene(sc, use_colors=use_colors, colors=colors, use_cov=use_cov, cov=cov).forward()
    leaf = {"means3D": sc.means3D.double().clone().requires_grad_(True),
            "opacities": sc.opacities.double().clone().requires_grad_(True)}
    kw = {}
    if use_colors:
        leaf["colors"] = colors.double().clone().requires_grad_(True)
        kw["colors_precomp"] = leaf["colors"]
    else:
        leaf["shs"] = sc.shs.double().clone().requires_grad_(True)
        kw["shs"] = leaf["shs"]
    if use_cov:
        leaf["cov"] = cov.double().clone().requires_grad_(True)
        kw["cov3D_precomp"] = leaf["cov"]
    else:
        leaf["scales"] = sc.scales.double().clone().requires_grad_(True)
        leaf["rotations"] = sc.rotations.double().clone().requires_grad_(True)
        kw["scales"], kw["rotations"] = leaf["scales"], leaf["rotations"]
    m2 = torch.zeros(sc.n, 3, dtype=torch.float64, requires_grad=True)
    r = TO.rasterize(cam.width, cam.height, cam.tanfovx, cam.tanfovy, sc.bg, 1.0, cam.viewmatrix, cam.projmatrix,
                     sc.sh_degree, cam.campos, leaf["means3D"], m2, leaf["opacities"], **kw)
    return o, r, leaf, m2


@pytest.mark.parametrize("seed,n,w,h", [(5, 400, 72, 56), (6, 800, 64, 64), (8, 300, 40, 90)])
def test_c_oracle_forward_matches_torch(seed, n, w, h):
    from cfgs import scenes
    sc = scenes.scene_small(n=n, width=w, height=h, seed=seed)
    o, r, _, _ = _both(sc)
    np.testing.assert_array_equal(r["radii"].numpy(), o.radii)
    assert (r["n_contrib"].numpy() == o.n_contrib).mean() >= 0.999
    assert np.abs(r["color"].detach().numpy() - o.color).max() <= 1e-5
    assert np.abs(r["alpha"].detach().numpy() - o.alpha).max() <= 1e-5
    assert np.abs(r["depth"].detach().numpy() - o.depth).max() <= 1e-4


@pytest.mark.parametrize("use_colors,use_cov", [(False, False), (True, True), (False, True)])
def test_c_oracle_backward_matches_autograd(use_colors, use_cov):
    from cfgs import scenes
    sc = scenes.scene_small(n=400, width=72, height=56, seed=5)
    o, r, leaf, m2 = _both(sc, use_colors=use_colors, use_cov=use_cov)
    rng = np.random.default_rng(0)
    H, W = sc.camera.height, sc.camera.width
    gc = torch.tensor(rng.standard_normal((3, H, W)))
    gd = torch.tensor(rng.standard_normal((1, H, W)))
    ga = torch.tensor(rng.standard_normal((1, H, W)))
    ((r["color"] * gc).sum() + (r["depth"] * gd).sum() + (r["alpha"] * ga).sum()).backward()
    g = o.backward(gc.float().numpy(), gd.float().numpy(), ga.float().numpy())
    assert_grad_close("means2D", g["means2D"], m2.grad, floor=0.1)
    assert_grad_close("opacity", g["opacity"], leaf["opacities"].grad, floor=0.1)
    assert_grad_close("means3D", g["means3D"], leaf["means3D"].grad, floor=0.1)
    if use_colors:
        assert_grad_close("colors", g["colors"], leaf["colors"].grad, floor=0.1)
    else:
        assert_grad_close("sh", g["sh"], leaf["shs"].grad, floor=0.1)
    if use_cov:
        assert_grad_close("cov3D", g["cov3D"], leaf["cov"].grad, floor=0.1)
    else:
        assert_grad_close("scales", g["scales"], leaf["scales"].grad, floor=0.1)
        assert_grad_close("rotations", g["rotations"], leaf["rotations"].grad, floor=0.1)


def test_oracle_backward_matches_finite_differences():
    """Central differences (float64 torch restatement, h = 1e-6) on a few parameters."""
    from cfgs import scenes
    from oracle import torch_oracle as TO
    sc = scenes.scene_small(n=60, width=48, height=48, seed=13)
    cam = sc.camera
    rng = np.random.default_rng(2)
    gc = torch.tensor(rng.standard_normal((3, 48, 48)))

    def loss(means):
        r = TO.rasterize(cam.width, cam.height, cam.tanfovx, cam.tanfovy, sc.bg, 1.0, cam.viewmatrix,
                         cam.projmatrix, 3, cam.campos, means, torch.zeros(sc.n, 3, dtype=torch.float64),
                         sc.opacities.double(), shs=sc.shs.double(), scales=sc.scales.double(),
                         rotations=sc.rotations.double())
        return (r["color"] * gc).sum()

    m = sc.means3D.double().clone().requires_grad_(True)
    loss(m).backward()
    h = 1e-6
    idx = [(i, k) for i in range(0, 60, 7) for k in range(3)]
    for i, k in idx:
        mp, mm = sc.means3D.double().clone(), sc.means3D.double().clone()
        mp[i, k] += h
        mm[i, k] -= h
        fd = (loss(mp) - loss(mm)).item() / (2 * h)
        assert abs(fd - m.grad[i, k].item()) <= 1e-4 * max(1.0, abs(fd)), (i, k, fd, m.grad[i, k].item())


def test_oracle_exp_accuracy():
    from oracle import c_oracle
    xs = np.concatenate([np.linspace(-104, 88, 20001), -np.logspace(-8, 2, 2000), [0.0, -0.0]]).astype(np.float32)
    worst = 0.0
    for x in xs:
        got = c_oracle.exp(float(x))
        want = math.exp(float(x))
        if want < 1.2e-38:  # subnormal results: absolute error
            assert abs(got - want) <= 2e-45 * 2
            continue
        ulp = np.spacing(np.float32(want))
        worst = max(worst, abs(got - want) / float(ulp))
    assert worst <= 2.0, worst
    assert c_oracle.exp(-200.0) == 0.0
    assert math.isinf(c_oracle.exp(100.0))


@pytest.mark.parametrize("seed,n,w,h", [(3, 2000, 100, 75), (4, 500, 33, 17)])
def test_c_oracle_keys_and_ranges_are_a_stable_sort(seed, n, w, h):
    """The oracle's binning is the published one: every (Gaussian, touched tile) pair in
    Gaussian order with the 64-bit key tile << 32 | depth bits, stably sorted by key; the
    tile ranges are the key boundaries. Rebuilt here in numpy from the oracle's own
    per-Gaussian outputs (rectangles, depths)."""
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    sc = scenes.scene_small(n=n, width=w, height=h, seed=seed)
    o = Oracle.from_scene(sc).forward()
    keys, gids = [], []
    for g in range(n):
        if o.radii[g] <= 0:
            continue
        x0, y0, x1, y1 = (int(v) for v in o.rect[g])
        dbits = int(np.float32(o.rgbd[g, 3]).view(np.uint32))
        for ty in range(y0, y1):
            for tx in range(x0, x1):
                keys.append(((ty * o.gx + tx) << 32) | dbits)
                gids.append(g)
    keys = np.array(keys, dtype=np.uint64)
    gids = np.array(gids, dtype=np.uint32)
    order = np.argsort(keys, kind="stable")
    assert o.K == len(keys)
    np.testing.assert_array_equal(o.keys, keys[order])
    np.testing.assert_array_equal(o.gid, gids[order])
    tiles = (keys[order] >> np.uint64(32)).astype(np.int64)
    want = np.searchsorted(tiles, np.arange(o.gx * o.gy + 1), side="left")
    np.testing.assert_array_equal(o.ranges.astype(np.int64), want)


def test_c_oracle_edge_scenes():
    """Empty input, every Gaussian behind the camera, and screen-filling Gaussians: the
    C oracle against the float64 restatement."""
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    empty = scenes.scene_small(n=0, width=33, height=17, seed=1)
    o = Oracle.from_scene(empty).forward()
    assert o.K == 0 and np.all(o.n_contrib == 0) and np.all(o.final_T == 1.0)
    np.testing.assert_array_equal(o.color, np.broadcast_to(empty.bg.numpy()[:, None, None], o.color.shape))

    behind = scenes.scene_small(n=200, width=48, height=40, seed=2)
    m = behind.means3D.clone()
    m[:, 2] = -m[:, 2].abs() - 1.0          # every centre behind the camera
    behind.means3D = m
    o = Oracle.from_scene(behind).forward()
    assert o.K == 0 and np.all(o.radii == 0)

    big = scenes.scene_small(n=300, width=64, height=48, seed=3)
    s = big.scales.clone()
    s[:4] = 0.8                              # a few Gaussians that cover every tile
    big.scales = s
    o, r, _, _ = _both(big)
    assert o.K >= 4 * o.gx * o.gy
    np.testing.assert_array_equal(r["radii"].numpy(), o.radii)
    assert np.abs(r["color"].detach().numpy() - o.color).max() <= 1e-5


def test_contribution_counts_match_a_direct_count():
    """oracle.error_bound.contribution_counts (the term counts of the any-order sum
    bound) equals a pixel-by-pixel count over the oracle's lists."""
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    from oracle.error_bound import contribution_counts
    sc = scenes.scene_small(n=800, width=70, height=50, seed=2)
    o = Oracle.from_scene(sc).forward()
    want = np.zeros(o.N)
    for py in range(o.H):
        for px in range(o.W):
            t = (py // 16) * o.gx + px // 16
            for c in range(int(o.n_contrib[py * o.W + px])):
                want[o.gid[o.ranges[t] + c]] += 1
    got = contribution_counts(o)
    np.testing.assert_array_equal(got, want)
    assert got.sum() == o.n_contrib.sum() > 0
