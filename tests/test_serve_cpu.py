"""Host-side pieces of the request server (cfgs/serve.py) on CPU: the Poisson request
stream, the per-solve HBM estimate used for admission, and the latency summary."""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch


def test_poisson_stream_rate_mix_and_order():
    from cfgs import serve
    s = serve.poisson_stream(200.0, 60.0, 0.9, 64, 1, seed=11)
    arrivals = np.array([r.arrival for r in s])
    assert np.all(np.diff(arrivals) > 0) and arrivals[-1] < 60.0
    assert abs(len(s) - 12000) < 4 * math.sqrt(12000)          # Poisson count, 4 sigma
    pose = [r for r in s if r.kind == "pose"]
    assert abs(len(pose) / len(s) - 0.9) < 0.02
    assert {r.payload for r in pose} <= set(range(64)) and len({r.payload for r in pose}) == 64
    assert all(r.payload == 0 for r in s if r.kind == "render")
    assert [r.rid for r in s] == list(range(len(s)))
    again = serve.poisson_stream(200.0, 60.0, 0.9, 64, 1, seed=11)
    assert [(r.kind, r.arrival, r.payload) for r in again] == [(r.kind, r.arrival, r.payload) for r in s]


def test_solve_bytes_counts_inputs_workspaces_and_images():
    from cfgs import serve
    n, h, w = 1000, 90, 160
    f = lambda *shape: torch.zeros(*shape)
    pl = serve.PosePayload(f(n, 3), f(n, 1), f(n, 1, 3), f(n, 3), f(n, 4), f(3, h, w), camera=None, sh_degree=0)
    assert pl.nbytes == 4 * (n * (3 + 1 + 3 + 3 + 4) + 3 * h * w)
    need = serve.solve_bytes(pl)
    assert need > pl.nbytes + n * 64                               # plus per-Gaussian and per-instance workspaces
    pl2 = serve.PosePayload(f(2 * n, 3), f(2 * n, 1), f(2 * n, 1, 3), f(2 * n, 3), f(2 * n, 4), f(3, h, w),
                            camera=None, sh_degree=0)
    assert serve.solve_bytes(pl2) > need                           # grows with the Gaussian count


@pytest.mark.filterwarnings("ignore:All-NaN slice encountered")  # the empty summary reports NaN latencies
def test_stats_summary_percentiles():
    from cfgs import serve
    st = serve.ServeStats()
    for i in range(100):
        r = serve.Request(i, "pose" if i % 10 else "render", float(i), 0)
        r.done = r.arrival + (i + 1) / 100.0
        st.completed.append(r)
    st.wall = 50.0
    st.admitted_peak = 7
    s = st.summary("x")
    assert s["completed"] == 100 and s["throughput_req_s"] == 2.0
    assert s["pose_solves_per_s"] == 1.8 and s["renders_per_s"] == 0.2
    lat = np.array([(i + 1) / 100.0 for i in range(100)])
    assert s["latency_p50_s"] == round(float(np.percentile(lat, 50)), 4)
    assert s["latency_p99_s"] == round(float(np.percentile(lat, 99)), 4)
    assert s["peak_active_solves"] == 7
    empty = serve.ServeStats().summary("y")
    assert empty["completed"] == 0 and math.isnan(empty["latency_p50_s"])


def _payload(n=500, h=18, w=32, deg=0):
    from cfgs import scenes, serve
    f = lambda *shape: torch.rand(*shape)
    cam = scenes.make_camera(w, h, 30.0, 30.0)
    return serve.PosePayload(f(n, 3), f(n, 1), f(n, (deg + 1) ** 2, 3), f(n, 3), f(n, 4), f(3, h, w), cam, deg)


def test_validate_payload_rejects_malformed_and_oversized_requests():
    """The server refuses, on arrival, what it could not serve; a well-formed request
    passes. (CF-3DGS stops on a NaN loss, trainer/losses.py:126-127: NaN inputs are
    refused up front.)"""
    from cfgs import serve
    ok = _payload()
    assert serve.validate_payload(ok) == ""
    cases = {
        "xyz shape": lambda p: setattr(p, "xyz", torch.rand(p.xyz.shape[0], 2)),
        "target size": lambda p: setattr(p, "target", torch.rand(3, 10, 10)),
        "opacity count": lambda p: setattr(p, "opacities", torch.rand(3, 1)),
        "sh width": lambda p: (setattr(p, "sh_degree", 2)),
        "sh degree": lambda p: setattr(p, "sh_degree", 5),
        "dtype": lambda p: setattr(p, "scales", p.scales.double()),
        "nan": lambda p: p.xyz.__setitem__((3, 1), float("nan")),
        "inf": lambda p: p.target.__setitem__((0, 0, 0), float("inf")),
        "empty": lambda p: setattr(p, "xyz", torch.rand(0, 3)),
        "missing": lambda p: setattr(p, "rotations", None),
    }
    for name, spoil in cases.items():
        p = _payload()
        spoil(p)
        assert serve.validate_payload(p) != "", name
    assert serve.validate_payload(ok, hbm_budget=serve.solve_bytes(ok)) == ""
    why = serve.validate_payload(ok, hbm_budget=serve.solve_bytes(ok) - 1)
    assert "HBM budget" in why


def test_cancel_is_thread_safe_and_recorded():
    import threading
    from cfgs import serve
    srv = serve.ContinuousBatchServer([], [], device="cpu", epoch=25, iters=300)
    ts = [threading.Thread(target=srv.cancel, args=(i,)) for i in range(50)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert all(srv._is_cancelled(i) for i in range(50)) and not srv._is_cancelled(50)
