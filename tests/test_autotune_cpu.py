"""Render-schedule autotuner host logic (cfgs/autotune.py) and the schedule C ABI's
argument checks; no GPU: candidates are timed by a fake measure."""
from __future__ import annotations

import json

import pytest


def test_schedule_abi_rejects_unsupported_shapes():
    from cfgs import autotune, native
    lib = native.load()
    S = native.RenderSchedule
    for bad in [(96, 4, 64), (64, 8, 64), (128, 6, 64), (128, 4, 48), (128, 4, 256), (0, 4, 64)]:
        assert lib.cfgs_render_schedule_check(native.C.byref(S(*bad, 0)), None) == 1
    assert lib.cfgs_render_schedule_check(None, None) == 1
    r = S()
    assert lib.cfgs_render_schedule_check(native.C.byref(S(0, 0, 0, 0)), native.C.byref(r)) == 0
    assert (r.fwd_batch, r.fwd_warps, r.bwd_batch) == (128, 4, 64)  # zeros: the default
    for good in [(64, 4, 32), (256, 8, 128), (128, 8, 64)]:
        assert lib.cfgs_render_schedule_check(native.C.byref(S(*good, 0)), native.C.byref(r)) == 0
        assert (r.fwd_batch, r.fwd_warps, r.bwd_batch) == good
    # the binning launch mode: 0 (per stage) or 1 (one persistent launch), kept as given
    assert lib.cfgs_render_schedule_check(native.C.byref(S(0, 0, 0, 1)), native.C.byref(r)) == 0
    assert (r.fwd_batch, r.fwd_warps, r.bwd_batch, r.bin_launch) == (128, 4, 64, 1)
    assert lib.cfgs_render_schedule_check(native.C.byref(S(64, 4, 32, 1)), native.C.byref(r)) == 0
    assert r.bin_launch == 1
    for bad_mode in (2, -1):
        assert lib.cfgs_render_schedule_check(native.C.byref(S(128, 4, 64, bad_mode)), None) == 1
    with pytest.raises(RuntimeError):
        autotune.set_schedule(autotune.Schedule(96, 4, 64))


def test_schedule_is_per_thread():
    """The host's current schedule belongs to the calling thread; the library keeps none
    (every call's settings carry it), so threads with different schedules do not mix."""
    import threading
    from cfgs import autotune, raster

    class RS:  # the fields make_settings reads
        image_height = image_width = 16
        tanfovx = tanfovy = 1.0
        bg = viewmatrix = projmatrix = campos = None
        scale_modifier = 1.0
        sh_degree = 0
        prefiltered = debug = False

    seen = {}

    def worker(name, sched):
        with autotune.using(sched):
            s = raster.make_settings(RS, [])
            seen[name] = (s.schedule.fwd_batch, s.schedule.fwd_warps, s.schedule.bwd_batch)

    assert autotune.get_schedule() == autotune.DEFAULT
    t1 = threading.Thread(target=worker, args=("a", autotune.Schedule(256, 8, 32)))
    t2 = threading.Thread(target=worker, args=("b", autotune.Schedule(64, 4, 128)))
    t1.start(), t2.start(), t1.join(), t2.join()
    assert seen == {"a": (256, 8, 32), "b": (64, 4, 128)}
    assert autotune.get_schedule() == autotune.DEFAULT  # this thread's is untouched
    s = raster.make_settings(RS, [], schedule=autotune.Schedule(128, 8, 64))
    assert (s.schedule.fwd_batch, s.schedule.fwd_warps) == (128, 8)


def test_default_schedule_is_the_hand_tuned_one():
    from cfgs import autotune
    assert autotune.DEFAULT == autotune.Schedule(128, 4, 64)
    assert (autotune.DEFAULT.fwd_batch, autotune.DEFAULT.fwd_warps) == autotune.FWD_CANDIDATES[0]
    assert autotune.DEFAULT.bwd_batch == autotune.BWD_CANDIDATES[0]


def test_pick_keeps_incumbent_within_margin():
    from cfgs.autotune import pick
    assert pick(["a", "b", "c"], {"a": 1.0, "b": 0.99, "c": 1.2}, 0.02) == "a"
    assert pick(["a", "b", "c"], {"a": 1.0, "b": 0.97, "c": 0.90}, 0.02) == "c"
    assert pick(["a", "b"], {"a": 1.0, "b": 0.97}, 0.0) == "b"


def test_buckets_and_keys():
    from cfgs.autotune import batch_key, bucket, raster_key
    assert [bucket(n) for n in (0, 1, 2, 3, 230400, 1 << 20)] == [1, 1, 2, 4, 262144, 1 << 20]
    assert raster_key(1_000_000, 1920, 1080, 16) == "raster/n1048576/1920x1080/m16"
    assert batch_key(230400, 920, 1) == "batch/n262144/t1024/m1"


def test_tune_coordinate_search_and_cache(tmp_path):
    from cfgs import autotune
    # a fake workload whose cost favours the 8-warp forward with batch 256 and a backward batch of 32
    cost = {(128, 4): 10.0, (64, 4): 10.5, (256, 4): 9.9, (128, 8): 8.0, (256, 8): 7.5}
    bcost = {64: 0.0, 32: -1.0, 128: 0.5}
    calls = []

    def measure(run, s):
        calls.append(s)
        return cost[(s.fwd_batch, s.fwd_warps)] + bcost[s.bwd_batch]

    path = tmp_path / "cache.json"
    t = autotune.Autotuner(path, measure=measure)
    s = t.tune("raster/n1/1x1/m1", run=lambda: None)
    assert s == autotune.Schedule(256, 8, 32)
    # 5 forward shapes at the default backward batch, 2 more backward batches, then the
    # interleaved confirmation (default, chosen) x 2
    assert len(calls) == 11 and all(c.bwd_batch == 64 for c in calls[:5])
    assert calls[7:] == [autotune.DEFAULT, s, autotune.DEFAULT, s]
    data = json.loads(path.read_text())
    (k, e), = data.items()
    assert k.endswith("|raster/n1/1x1/m1") and e["schedule"] == {"fwd_batch": 256, "fwd_warps": 8, "bwd_batch": 32,
                                                                 "bin_launch": 0}
    assert e["ms"]["256/8/32"] == pytest.approx(6.5)
    # a second tuner on the same file answers from the cache without measuring
    calls.clear()
    t2 = autotune.Autotuner(path, measure=measure)
    assert t2.tune("raster/n1/1x1/m1", run=lambda: None) == s and not calls
    assert t2.tune("raster/n1/1x1/m1", run=lambda: None, force=True) == s and len(calls) == 11


def test_confirmation_rejects_a_noisy_winner(tmp_path):
    from cfgs import autotune
    seen = {}

    def measure(run, s):  # the 64-batch forward looks fast once, then no longer
        n = seen.get(s, 0)
        seen[s] = n + 1
        if s.fwd_batch == 64 and n == 0:
            return 9.0
        return 10.0

    t = autotune.Autotuner(tmp_path / "c.json", measure=measure)
    assert t.tune("k", run=lambda: None) == autotune.DEFAULT


def test_unreadable_cache_is_ignored(tmp_path):
    from cfgs import autotune
    p = tmp_path / "c.json"
    p.write_text("{not json")
    t = autotune.Autotuner(p, measure=lambda run, s: 1.0)
    assert t.lookup("x") is None
    assert t.tune("x", run=lambda: None) == autotune.DEFAULT  # all equal: the default stays
    assert json.loads(p.read_text())
