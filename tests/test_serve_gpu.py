"""Continuous-batching server on the GPU: requests arriving while others run are
admitted at epoch boundaries, several solves share the device, renders overlap, and
every result equals the same request served alone."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import pose, scenes, serve
    payloads, probs = [], []
    for (w, h, n, sd) in [(96, 54, None, 2), (128, 72, 6000, 3), (80, 48, 3000, 4), (112, 64, None, 5)]:
        sc = scenes.scene_pose(width=w, height=h, n=n, seed=sd)
        p = pose.make_problem(sc, DEV)
        probs.append(p)
        payloads.append(serve.payload_from_problem(p, sc.camera))
    target = serve.RenderTarget(scenes.scene_small(n=4096, width=128, height=96, seed=9), DEV)
    return serve, pose, payloads, probs, [target]


def _stream(serve, kinds_payloads, spacing):
    return [serve.Request(i, k, i * spacing, p) for i, (k, p) in enumerate(kinds_payloads)]


ITERS, EPOCH = 40, 10


def test_results_equal_alone_and_overlap(setup):
    serve, pose, payloads, probs, targets = setup
    reqs = _stream(serve, [("pose", 0), ("pose", 1), ("render", 0), ("pose", 2), ("pose", 3), ("render", 0),
                           ("pose", 1)], spacing=0.001)
    srv = serve.ContinuousBatchServer(payloads, targets, DEV, max_slots=8, epoch=EPOCH, iters=ITERS)
    st = srv.run(reqs)
    assert len(st.completed) == len(reqs)
    assert st.admitted_peak >= 2
    alone = {i: pose.solve(p, iters=ITERS, mode="fused")[0] for i, p in enumerate(probs)}
    want_img = float(targets[0].render().double().sum())
    for r in reqs:
        if r.kind == "pose":
            assert np.array_equal(np.float32(r.result), np.float32(alone[r.payload])), r.rid
        else:
            assert r.result == want_img
        assert r.done >= r.arrival


def test_hbm_budget_limits_admission(setup):
    serve, pose, payloads, probs, targets = setup
    reqs = _stream(serve, [("pose", 0), ("pose", 1), ("pose", 2)], spacing=0.0)
    one = serve.solve_bytes(payloads[1]) + 1
    srv = serve.ContinuousBatchServer(payloads, targets, DEV, max_slots=8, hbm_budget=one, epoch=EPOCH, iters=ITERS)
    st = srv.run(reqs)
    assert len(st.completed) == 3 and st.admitted_peak == 1
    for r in reqs:
        xi, _ = pose.solve(probs[r.payload], iters=ITERS, mode="fused")
        assert np.array_equal(np.float32(r.result), np.float32(xi))


def test_plain_fifo_server_runs(setup):
    serve, pose, payloads, probs, targets = setup
    reqs = _stream(serve, [("pose", 0), ("render", 0), ("pose", 2)], spacing=0.0)
    st = serve.PlainFifoServer(payloads, targets, DEV, iters=ITERS).run(reqs)
    s = st.summary("plain")
    assert s["completed"] == 3 and s["latency_p99_s"] >= s["latency_p50_s"] > 0
