"""Batched pose solves on the GPU: every solve in a batch ends bit-identical to the same
solve run alone on the single-solve fused path, and to the same solve in a different
mix; an undersized instance capacity is detected and retried."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import batch, pose, scenes
    return batch, pose, scenes


def _problems(pose, scenes, specs):
    return [pose.make_problem(scenes.scene_pose(width=w, height=h, n=n, seed=sd), DEV) for (w, h, n, sd) in specs]


SPECS = [(160, 90, None, 2), (128, 72, 5000, 7), (96, 54, 9000, 11)]


def test_batch_matches_single_fused_solves(mods):
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, SPECS)
    iters = 60
    res = batch.BatchSolver(probs, graph_chunk=20).solve(iters)
    assert not res.overflowed
    for s, p in enumerate(probs):
        xi_single, _ = pose.solve(p, iters=iters, mode="fused")
        assert np.array_equal(res.xi[s].astype(np.float32), xi_single.astype(np.float32)), (s, res.xi[s], xi_single)


def test_alone_equals_in_mix(mods):
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, SPECS)
    iters = 40
    mix = batch.BatchSolver(probs, use_graph=False).solve(iters)
    alone = batch.BatchSolver([probs[1]], use_graph=False).solve(iters)
    swapped = batch.BatchSolver([probs[2], probs[1]], use_graph=False).solve(iters)
    assert np.array_equal(mix.xi[1], alone.xi[0])
    assert np.array_equal(mix.xi[1], swapped.xi[1])
    assert np.array_equal(mix.xi[2], swapped.xi[0])


def test_graph_replay_equals_direct_launches(mods):
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, SPECS[:2])
    a = batch.BatchSolver(probs, use_graph=True, graph_chunk=10).solve(30)
    b = batch.BatchSolver(probs, use_graph=False).solve(30)
    assert np.array_equal(a.xi, b.xi)


def test_capacity_overflow_is_detected_and_retried(mods):
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, SPECS[:2])
    ok = batch.BatchSolver(probs, use_graph=False).solve(20)
    small = batch.BatchSolver(probs, use_graph=False, capacity_factor=0.3)
    r = small.solve(20)
    assert r.retries >= 1 and not r.overflowed
    assert np.array_equal(r.xi, ok.xi)


def test_batch_solve_recovers_pose(mods):
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, [(320, 180, None, 4), (320, 180, 40000, 5)])
    res = batch.BatchSolver(probs).solve(300)
    for s, p in enumerate(probs):
        e0 = pose.pose_error(np.zeros(6), p.xi_gt)
        e1 = pose.pose_error(res.xi[s], p.xi_gt)
        assert e1[0] < 0.25 * e0[0] + 0.01 and e1[1] < 0.25 * e0[1] + 1e-3, (s, e0, e1)


def test_prepare_and_iterate_equal_solve(mods):
    """The eager interface (prepare() + iterate()) takes the same steps as solve()."""
    batch, pose, scenes = mods
    probs = _problems(pose, scenes, SPECS[:2])
    ref = batch.BatchSolver(probs, use_graph=False).solve(15).xi
    bs = batch.BatchSolver(probs, use_graph=False)
    args = bs.prepare()
    for _ in range(15):
        bs.iterate(args)
    torch.cuda.synchronize()
    assert np.array_equal(bs.xi.double().cpu().numpy(), ref)


def test_one_launch_binning_equals_per_stage_launches(mods):
    """The binning as one persistent cooperative launch (schedule bin_launch=1) gives the
    per-stage launches' results bit for bit: through CUDA-graph replays, in direct
    launches, with a large batch (the emission's offsets from the rank-sum scan), and
    when an undersized capacity overflows and is retried."""
    batch, pose, scenes = mods
    from cfgs import autotune
    probs = _problems(pose, scenes, SPECS)
    one = autotune.Schedule(bin_launch=1)
    ref = batch.BatchSolver(probs, use_graph=False).solve(25)
    with autotune.using(one):
        graphed = batch.BatchSolver(probs, graph_chunk=10).solve(25)
        direct = batch.BatchSolver(probs, use_graph=False).solve(25)
        small = batch.BatchSolver(probs, use_graph=False, capacity_factor=0.3).solve(25)
    for r in (graphed, direct, small):
        assert not r.overflowed
        assert np.array_equal(r.xi, ref.xi)
    big = _problems(pose, scenes, [(640, 360, 600_000, 3), (960, 540, 1_000_000, 5), (960, 540, 900_000, 9)])
    ref_big = batch.BatchSolver(big, use_graph=False).solve(3)
    with autotune.using(one):
        one_big = batch.BatchSolver(big, use_graph=False).solve(3)
    assert np.array_equal(one_big.xi, ref_big.xi)
