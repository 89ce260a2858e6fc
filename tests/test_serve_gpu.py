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


def test_failures_are_confined_to_their_requests(setup):
    """Host-side fault injection (no device fault): a malformed request and one larger
    than the HBM budget are rejected on arrival, a queued and a running solve are
    cancelled, a simulated device allocation failure fails its request, and a solve
    whose pose is poisoned with NaN mid-run is stopped and failed. Every other request
    ends with the result it has alone."""
    import copy
    serve, pose, payloads, probs, targets = setup
    from cfgs import scenes
    bad = copy.copy(payloads[0])
    bad.xyz = bad.xyz.clone()
    bad.xyz[5, 1] = float("nan")
    big_sc = scenes.scene_pose(width=256, height=144, seed=8)
    big = serve.payload_from_problem(pose.make_problem(big_sc, DEV), big_sc.camera)
    budget = 2 * max(serve.solve_bytes(p) for p in payloads)
    assert serve.solve_bytes(big) > budget
    pls = payloads + [bad, big]
    kinds = [("pose", 0), ("pose", 4), ("pose", 1), ("pose", 2), ("pose", 5), ("pose", 3), ("render", 0),
             ("pose", 1), ("pose", 0), ("render", 7)]
    reqs = _stream(serve, kinds, spacing=0.0)
    OOM_RID, NAN_RID, CANCEL_RUNNING, CANCEL_QUEUED = 3, 5, 2, 7
    seen = {"epochs": 0}

    def on_upload(req):
        if req.rid == OOM_RID:
            raise torch.cuda.OutOfMemoryError("simulated allocation failure")

    def on_epoch(bs, active):
        seen["epochs"] += 1
        rids = [r.rid for r in active]
        if seen["epochs"] == 2 and NAN_RID in rids:
            bs.xi[rids.index(NAN_RID)] = float("nan")
        if seen["epochs"] == 1:
            srv.cancel(CANCEL_RUNNING)

    srv = serve.ContinuousBatchServer(pls, targets, DEV, max_slots=3, hbm_budget=budget, epoch=EPOCH, iters=ITERS,
                                      hooks={"upload": on_upload, "epoch": on_epoch})
    srv.cancel(CANCEL_QUEUED)
    st = srv.run(reqs)
    status = {r.rid: r.status for r in reqs}
    assert status == {0: "ok", 1: "rejected", 2: "cancelled", 3: "failed", 4: "rejected", 5: "failed",
                      6: "ok", 7: "cancelled", 8: "ok", 9: "rejected"}, {r.rid: (r.status, r.error) for r in reqs}
    assert "non-finite" in reqs[NAN_RID].error and "allocation" in reqs[OOM_RID].error
    assert "HBM budget" in reqs[4].error
    s = st.summary("x")
    assert (s["completed"], s["rejected"], s["cancelled"], s["failed"]) == (3, 3, 2, 2)
    want = pose.solve(probs[0], iters=ITERS, mode="fused")[0]
    for rid in (0, 8):
        assert np.array_equal(np.float32(reqs[rid].result), np.float32(want)), rid
    assert reqs[6].result == float(targets[0].render().double().sum())
