"""Every render schedule (CfgsRenderSchedule, carried by each call: forward staging batch
and warps per tile, backward staging batch) gives bit-identical results: forward images, contributor
counts and final transmittances, every gradient of the drop-in rasteriser, and the
poses of batched solves. The autotuner picks among them on the GPU and caches the
choice."""
from __future__ import annotations

import itertools

import numpy as np
import pytest
import torch

from helpers import settings_for

pytestmark = pytest.mark.gpu
DEV = "cuda"

SCHEDULES = [(fb, fw, bb) for (fb, fw), bb in itertools.product([(128, 4), (64, 4), (256, 4), (128, 8), (256, 8)],
                                                                  [64, 32, 128])]


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as dgr
    from cfgs import autotune, raster, scenes
    return dgr, autotune, raster, scenes


def _run(dgr, raster, scene, depth_grads):
    rs = settings_for(dgr, scene)
    s = scene.to(DEV)
    torch.cuda.current_stream().synchronize()
    color, radii, depth, alpha, st = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations,
                                                    None)
    v = raster.inspect_state(st, scene.camera.width, scene.camera.height)
    g = torch.Generator().manual_seed(1)
    H, W = scene.camera.height, scene.camera.width
    gc = torch.randn(3, H, W, generator=g).to(DEV)
    gd = (torch.randn(1, H, W, generator=g) * 1e-3).to(DEV) if depth_grads else None
    ga = (torch.randn(1, H, W, generator=g) * 1e-3).to(DEV) if depth_grads else None
    grads = raster.backward(rs, st, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None, gc, gd, ga)
    torch.cuda.synchronize()
    out = {"color": color, "depth": depth, "alpha": alpha, "radii": radii, "n_contrib": v["n_contrib"].clone(),
           "final_T": v["final_T"].clone()}
    for i, t in enumerate(grads):
        if isinstance(t, torch.Tensor):
            out[f"grad{i}"] = t
    return {k: t.detach().clone() for k, t in out.items()}


@pytest.mark.parametrize("case", ["config0", "odd_size"])
@pytest.mark.parametrize("depth_grads", [False, True])
def test_every_schedule_is_bit_identical(mods, case, depth_grads):
    dgr, autotune, raster, scenes = mods
    sc = scenes.scene_small(n=16384, width=256, height=256, seed=0) if case == "config0" else \
        scenes.scene_small(n=2500, width=100, height=75, seed=7)
    with autotune.using(autotune.DEFAULT):
        ref = _run(dgr, raster, sc, depth_grads)
    assert ref["n_contrib"].max() > 0
    for sched in SCHEDULES:
        with autotune.using(autotune.Schedule(*sched)):
            out = _run(dgr, raster, sc, depth_grads)
        for k in ref:
            assert torch.equal(out[k], ref[k]), (sched, k)


def test_batched_solves_identical_under_every_forward_shape(mods):
    dgr, autotune, raster, scenes = mods
    from cfgs import batch, pose
    probs = [pose.make_problem(scenes.scene_pose(width=w, height=h, n=n, seed=sd), DEV)
             for (w, h, n, sd) in [(160, 90, None, 2), (128, 72, 5000, 7)]]
    with autotune.using(autotune.DEFAULT):
        ref = batch.BatchSolver(probs, use_graph=False).solve(20).xi
    for sched in [(256, 8, 32), (128, 8, 128), (64, 4, 32)]:
        with autotune.using(autotune.Schedule(*sched)):
            xi = batch.BatchSolver(probs, use_graph=False).solve(20).xi
        assert np.array_equal(xi, ref), sched


def test_autotuned_batch_matches_default(mods, tmp_path):
    dgr, autotune, raster, scenes = mods
    from cfgs import batch, pose
    probs = [pose.make_problem(scenes.scene_pose(width=160, height=90, seed=3), DEV)]
    with autotune.using(autotune.DEFAULT):
        ref = batch.BatchSolver(probs).solve(50).xi
        tuner = autotune.Autotuner(tmp_path / "cache.json")
        bs = batch.BatchSolver(probs, autotune=tuner)
        got = bs.solve(50).xi
        assert bs.schedule is not None
        assert tuner.lookup(autotune.batch_key(int(probs[0].xyz.shape[0]), bs.plan.num_tiles, bs.M)) == bs.schedule
    assert np.array_equal(got, ref)


def test_threads_with_different_schedules_concurrently(mods):
    """Two threads render two different workloads at the same time, each on its own
    stream under its own schedule (the library keeps none; each call carries the
    calling thread's): every result equals that workload's single-threaded result."""
    import threading
    dgr, autotune, raster, scenes = mods
    work = {"a": (scenes.scene_small(n=16384, width=256, height=256, seed=0), autotune.Schedule(256, 8, 32)),
            "b": (scenes.scene_small(n=2500, width=100, height=75, seed=7), autotune.Schedule(64, 4, 128))}
    with autotune.using(autotune.DEFAULT):
        ref = {k: _run(dgr, raster, sc, True) for k, (sc, _) in work.items()}
    results, errors = {k: [] for k in work}, []
    start = threading.Barrier(len(work))

    def worker(name):
        try:
            sc, sched = work[name]
            with torch.cuda.stream(torch.cuda.Stream()), autotune.using(sched):
                start.wait()
                for _ in range(4):
                    assert autotune.get_schedule() == sched
                    results[name].append(_run(dgr, raster, sc, True))
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(k,)) for k in work]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for name in work:
        assert len(results[name]) == 4
        for out in results[name]:
            for k in ref[name]:
                assert torch.equal(out[k], ref[name][k]), (name, k)
