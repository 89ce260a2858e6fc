"""bench.py's multi-rank logic on CPU: N > 1 runs independent replicas (the path does not
shard), the job time is the slowest rank's (a MAX all-reduce over the default process
group, here gloo with world size 2), the value is the units of all ranks over that time,
and the reference arm runs on rank 0 only."""
from __future__ import annotations

import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = 10.0 * (rank + 1)  # rank 1 is the slow one
        job = bench.max_over_ranks(local, world, torch.device("cpu"))
        out.put((rank, job, bench.job_rate(world, 5, job / 1000.0)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [20.0, 20.0]            # both ranks see the slowest time
    assert res[0][2] == pytest.approx(2 * 5 / 0.020)      # all ranks' units over it


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, None) == 3.5
    assert bench.job_rate(1, 4, 2.0) == 2.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
