"""Frame initialisation on the GPU against the C oracle (oracle/pointcloud_oracle.c):
unprojection, three-nearest-neighbour mean squared distance and voxel down-sampling
are integer/float work with one fixed rounding sequence, so the outputs must agree
bit for bit (voxels in the same order)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import bits

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def pc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cfgs import pointcloud
    return pointcloud


def test_depth_to_points_bit_exact(pc):
    from oracle import c_oracle
    rng = np.random.default_rng(0)
    d = rng.uniform(0.2, 10.0, (37, 61)).astype(np.float32)
    K = np.array([[52.5, 0, 30.2], [0, 49.75, 18.6], [0, 0, 1]])
    got = pc.depth_to_points(torch.tensor(d, device=DEV), K).cpu().numpy()
    want = c_oracle.depth_to_points(d, np.float32(52.5), np.float32(49.75), np.float32(30.2), np.float32(18.6))
    np.testing.assert_array_equal(bits(got), bits(want))


def _clouds():
    rng = np.random.default_rng(3)
    out = {"normal": rng.normal(0, 1, (20000, 3)).astype(np.float32)}
    c = rng.normal(0, 0.01, (9000, 3)).astype(np.float32)
    c[:3000] += np.float32(5.0)
    c[4000:4050] = c[10]  # exact duplicates
    out["clusters_dups"] = c
    # a depth-map surface, as the pose path produces
    v, u = np.mgrid[0:90, 0:160].astype(np.float32)
    d = (2.0 + np.sin(u / 13.0) + 0.5 * np.cos(v / 7.0)).astype(np.float32)
    out["surface"] = np.stack([(u - 80) / 120 * d, (v - 45) / 120 * d, d], -1).reshape(-1, 3).astype(np.float32)
    for k in (1, 2, 3, 4):
        out[f"tiny{k}"] = rng.normal(0, 1, (k, 3)).astype(np.float32)
    return out


@pytest.mark.parametrize("name", list(_clouds().keys()))
def test_knn3_bit_exact(pc, name):
    from oracle import c_oracle
    p = _clouds()[name]
    got = pc.dist_cuda2(torch.tensor(p, device=DEV)).cpu().numpy()
    want = c_oracle.knn3_mean_dist2(p)
    np.testing.assert_array_equal(bits(got), bits(want))


@pytest.mark.parametrize("case", ["unit", "wide_grid", "no_colour"])
def test_voxel_down_sample_bit_exact(pc, case):
    from oracle import c_oracle
    rng = np.random.default_rng(4)
    if case == "wide_grid":  # more than 2^32 cells: the two-round key sort
        p = rng.uniform(-100, 100, (30000, 3)).astype(np.float32)
        p[:2000] = (p[:1] + rng.uniform(0, 0.02, (2000, 3))).astype(np.float32)
        s = 0.01
    else:
        p = rng.normal(0, 0.2, (50000, 3)).astype(np.float32)
        s = 0.01
    col = None if case == "no_colour" else rng.uniform(0, 1, (len(p), 3)).astype(np.float32)
    gp, gc = pc.voxel_down_sample(torch.tensor(p, device=DEV), None if col is None else torch.tensor(col, device=DEV),
                                  s)
    wp, wc = c_oracle.voxel_down_sample(p, col, s)
    assert gp.shape[0] == wp.shape[0] and wp.shape[0] < len(p)
    np.testing.assert_array_equal(bits(gp.cpu().numpy()), bits(wp))
    if col is not None:
        np.testing.assert_array_equal(bits(gc.cpu().numpy()), bits(wc))


def test_gaussians_from_points(pc):
    """create_from_pcd (scene/gaussian_model_cf.py:175-210) on a down-sampled surface."""
    from oracle import c_oracle
    p = _clouds()["surface"]
    col = np.random.default_rng(5).uniform(0, 1, p.shape).astype(np.float32)
    g = pc.gaussians_from_points(torch.tensor(p, device=DEV), torch.tensor(col, device=DEV), sh_degree=3)
    d2 = np.maximum(c_oracle.knn3_mean_dist2(p), np.float32(1e-7))
    want = np.log(np.sqrt(torch.tensor(d2).numpy()))
    np.testing.assert_allclose(g["scaling"][:, 0].cpu().numpy(), want, rtol=0, atol=1e-6)
    assert g["features_dc"].shape == (len(p), 1, 3) and g["features_rest"].shape == (len(p), 15, 3)
    np.testing.assert_array_equal(g["features_dc"][:, 0].cpu().numpy(), col)
    assert torch.all(g["rotation"][:, 0] == 1) and torch.allclose(torch.sigmoid(g["opacity"]), torch.tensor(0.1))
