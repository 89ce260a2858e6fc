"""CPU checks of the frame-initialisation oracle (oracle/pointcloud_oracle.c) against
independent formulations: scipy's k-d tree for the three nearest neighbours, numpy for
the unprojection and a dictionary-of-voxels restatement of Open3D's down-sampling."""
from __future__ import annotations

import numpy as np
import pytest


def test_depth_to_points_oracle_matches_numpy():
    from oracle import c_oracle
    rng = np.random.default_rng(0)
    d = rng.uniform(0.5, 8.0, (13, 17)).astype(np.float32)
    fx, fy, cx, cy = np.float32(21.5), np.float32(19.25), np.float32(8.3), np.float32(6.1)
    got = c_oracle.depth_to_points(d, fx, fy, cx, cy)
    v, u = np.mgrid[0:13, 0:17].astype(np.float32)
    want = np.stack([((u - cx) / fx) * d, ((v - cy) / fy) * d, d], -1).reshape(-1, 3)
    np.testing.assert_array_equal(got, want)


def test_knn_oracle_matches_kdtree():
    spatial = pytest.importorskip("scipy.spatial")
    from oracle import c_oracle
    rng = np.random.default_rng(1)
    p = rng.normal(0, 1, (3000, 3)).astype(np.float32)
    p[100:110] = p[5]  # duplicates: zero distances
    got = c_oracle.knn3_mean_dist2(p)
    dist, _ = spatial.cKDTree(p.astype(np.float64)).query(p.astype(np.float64), k=4)
    # k-d tree distances include the point itself (0) and, for duplicates, its twins
    want = (dist[:, 1:4] ** 2).mean(1)
    assert np.abs(got - want).max() <= 1e-5 * max(1.0, np.abs(want).max())


def test_voxel_oracle_matches_dict_restatement():
    from oracle import c_oracle
    rng = np.random.default_rng(2)
    p = rng.uniform(-0.3, 0.3, (5000, 3)).astype(np.float32)
    c = rng.uniform(0, 1, (5000, 3)).astype(np.float32)
    s = 0.05
    gp, gc = c_oracle.voxel_down_sample(p, c, s)
    mn = p.min(0).astype(np.float64) - 0.5 * s
    vox = {}
    for i in range(len(p)):
        k = tuple(np.floor((p[i].astype(np.float64) - mn) / s).astype(np.int64))
        acc = vox.setdefault(k, [np.zeros(3), np.zeros(3), 0])
        for a in range(3):  # input order, float64, as Open3D's AccumulatedPoint
            acc[0][a] += float(p[i, a])
            acc[1][a] += float(c[i, a])
        acc[2] += 1
    keys = sorted(vox)
    want_p = np.array([vox[k][0] / vox[k][2] for k in keys], np.float32)
    want_c = np.array([vox[k][1] / vox[k][2] for k in keys], np.float32)
    np.testing.assert_array_equal(gp, want_p)
    np.testing.assert_array_equal(gc, want_c)
