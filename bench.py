#!/usr/bin/env python
"""Benchmark of the rasteriser hot path: forward + L1 loss + backward of 1,000,000 SH
degree-3 Gaussians at 1920x1080 (synthetic scene with the workload's shapes and value
distributions; the reference's datasets are not available).

`python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]`
prints one JSON line. N > 1 runs N independent replicas under torchrun (the path does
not shard: no collective), value = total iterations/s over all ranks.

--impl reference times the reference algorithm's CPU implementation (the oracle port,
C + OpenMP on every host core) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "cf-3dgs_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "fwd+bwd iters/s at 1M Gaussians 1080p"
UNIT = "iters/s"


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest of the ranks' values (the slowest rank's time); x itself for one rank.
    Every rank must call it (a collective on the default process group)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, steps: int, seconds: float) -> float:
    """Whole-job throughput: every rank runs `steps` units; the job takes the slowest
    rank's time."""
    return world * steps / seconds


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=1_000_000)
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-pose", action="store_true", help="skip the pose-solve half of the metric")
    p.add_argument("--no-tune", action="store_true", help="keep the default render schedule (no autotuning)")
    p.add_argument("--no-plain", action="store_true", help="skip the plain GPU path's iteration")
    p.add_argument("--bin-launch", type=int, default=0, choices=[0, 1],
                   help="pose_iter/batch_iter: binning as one launch per stage (0) or one persistent launch (1)")
    p.add_argument("--cpu-budget-s", type=float, default=20.0)
    p.add_argument("--workload", default="fwdbwd",
                   choices=["fwdbwd", "plain", "pose", "pose_iter", "batch", "batch_iter", "serve", "ssim", "init",
                            "optim"])
    p.add_argument("--serve-rate", type=float, default=200.0)
    p.add_argument("--serve-seconds", type=float, default=60.0)
    p.add_argument("--serve-slots", type=int, default=64)
    return p.parse_args()


def bench_config(sc, K: int, world: int) -> dict:
    """The workload description both arms print (the same dict for the same workload)."""
    D = (sc.sh_degree + 1) ** 2
    return {"workload": f"{sc.n} SH{sc.sh_degree} Gaussians, {sc.camera.width}x{sc.camera.height}, "
                        "fwd + L1 loss + bwd", "num_rendered": int(K),
            "l2": f"inputs larger than L2 (Gaussian parameters {sc.n * (44 + 12 * D) / 1e6:.0f} MB)",
            "parallelism": "replicas" if world > 1 else "1 GPU"}


def _cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# Algorithmic bytes of one fwd + bwd iteration of the published algorithm, item by item
# (N Gaussians, K tile instances, HW pixels, T tiles, D SH coefficients): the arrays it
# must read and write once. Grouped by this build's phases; the binning group (12K
# duplicate write + 24K one logical sort read+write + 8K + 8T ranges) covers the depth
# sort and the instance binning together.
# ---------------------------------------------------------------------------
def phase_bytes(N: int, K: int, HW: int, D: int, T: int) -> dict:
    params = N * (44 + 12 * D)
    return {
        "preprocess": params + 48 * N + 8 * N,                 # parameters read, geometry write, scan
        "binning": 12 * K + 24 * K + 8 * K + 8 * T,            # duplicate, sort, tile ranges
        "composite": 44 * K + 28 * HW,
        "render_bwd": 44 * K + 28 * HW + 36 * N,               # + the per-Gaussian 2D gradients written
        "preprocess_bwd": N * (44 + 12 * D + 48 + 36) + N * (44 + 12 * D + 24),
    }


# Bytes this build's render backward moves by design on top of the algorithm's: one
# 48-byte gradient record per kept instance (written, then read by the preprocess
# backward) and the one-byte written marks.
def render_bwd_design_bytes(K: int, kept: int) -> int:
    return 48 * kept + K


# FP32 floating-point operations per plain-algorithm evaluation (E = sum of the per-pixel
# contributor counts), counted with ncu (sm__sass_thread_inst_executed_op_{ffma,fadd,
# fmul,ffma2,fadd2,fmul2}_pred_on.sum: FFMA 2, FADD/FMUL 1, FFMA2 4, FADD2/FMUL2 2 flops)
# on the render kernels of a 250,000-Gaussian scene with the benchmark's distributions at
# 1920x1080 (E = 634M): forward 5.24e9 and backward 8.46e9 flops per launch.
FLOPS_PER_EVAL = {"composite": 5.24e9 / 633965142, "render_bwd": 8.46e9 / 633965142}


def alu_roofline(E: int, phase_ms: dict, pb: dict, peaks: dict) -> dict:
    """FP32 roofline of the two render kernels: E x counted flops per evaluation over the
    kernel time against the nominal FP32 peak (SMs x 128 lanes x 2 flops x max clock; no
    measured FP32 peak is available). Also the iteration's lower bound with each phase at
    its tighter bound (bytes / HBM or flops / FP32) against the measured phases."""
    import torch
    props = torch.cuda.get_device_properties(0)
    mhz = peaks.get("sm_max_mhz") or 2070.0
    peak = props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12
    out = {"E": E, "fp32_peak_tflops": round(peak, 2), "peak_source": "nominal (SMs x 128 x 2 x max clock)",
           "flops_per_eval": {k: round(v, 3) for k, v in FLOPS_PER_EVAL.items()},
           "flops_source": "ncu-counted FP32 instructions of the render kernels (250k-Gaussian scene, same "
                           "distributions), per plain-algorithm evaluation"}
    t_min = 0.0
    for k, ms in phase_ms.items():
        t_hbm = pb[k] / (peaks["hbm_gbs"] * 1e9)
        t_alu = E * FLOPS_PER_EVAL[k] / (peak * 1e12) if k in FLOPS_PER_EVAL else 0.0
        t_min += max(t_hbm, t_alu)
        if k in FLOPS_PER_EVAL:
            tf = E * FLOPS_PER_EVAL[k] / (ms / 1000.0) / 1e12
            out[k] = {"achieved_tflops": round(tf, 3), "frac": round(tf / peak, 4)}
    out["iteration_bound_ms"] = round(t_min * 1000.0, 4)
    out["iteration_frac"] = round(t_min * 1000.0 / sum(phase_ms.values()), 4)
    return out


def _peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured", "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0))}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback", "sm_max_mhz": 2070.0}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
# capture of the 1M-Gaussian 1080p workload (metrics that take one pass), at the
# instance count K it was taken at; scaled by instances for another K.
NCU_TRAFFIC = {"render_bwd": (177717504 + 80580864, 12433348),
               "composite": (67001088 + 30771968, 12433348),
               "preprocess_bwd": (452126720 + 293896704, 12433348)}


def _traffic(kernel: str, K: int):
    if kernel not in NCU_TRAFFIC:
        return None
    b, k0 = NCU_TRAFFIC[kernel]
    return int(b * K / k0)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(a) -> None:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    import diff_gaussian_rasterization as dgr
    from cfgs import raster, scenes

    sc = scenes.scene_large(n=a.n, width=a.width, height=a.height, seed=1)
    cam = sc.camera.to(dev)
    rs = dgr.GaussianRasterizationSettings(cam.height, cam.width, cam.tanfovx, cam.tanfovy, sc.bg.to(dev), 1.0,
                                           cam.viewmatrix, cam.projmatrix, sc.sh_degree, cam.campos, False, False)
    s = sc.to(dev)
    target = s.target
    HW = cam.width * cam.height

    from cfgs import autotune
    from cfgs.loss import l1_loss_and_grad
    if a.no_tune:
        sched = autotune.DEFAULT
        autotune.set_schedule(sched)
    else:
        sched = autotune.tune_rasterizer(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None,
                                         tuner=autotune.Autotuner())
    loss_buf = torch.empty((), dtype=torch.float32, device=dev)
    grad_buf = torch.empty_like(target)
    loss_scratch = torch.empty(4096, dtype=torch.uint8, device=dev)

    last_state = [None]

    def step(timers=None):
        color, radii, depth, alpha, st = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales,
                                                        s.rotations, None, timers=timers)
        # L1 of the clamped render and its gradient in one fused pass
        loss, g = l1_loss_and_grad(color, target, clamp=True, out=loss_buf, grad_out=grad_buf, scratch=loss_scratch)
        raster.backward(rs, st, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None, g, None, None,
                        timers=timers)
        last_state[0] = st
        return loss, st.num_rendered

    for _ in range(max(a.warmup, 0)):
        step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    timers: dict = {}
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    barrier()
    t0.record()
    K = 0
    for _ in range(a.steps):
        _, K = step(timers)
    t1.record()
    barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(t0.elapsed_time(t1), world, dev)
    ms_per_step = total_ms / a.steps
    value = job_rate(world, a.steps, total_ms / 1000.0)

    phase_ms = {k: sum(s_.elapsed_time(e_) for s_, e_ in v) / len(v) for k, v in timers.items()}
    D = (sc.sh_degree + 1) ** 2
    T = ((cam.width + 15) // 16) * ((cam.height + 15) // 16)
    pb = phase_bytes(sc.n, K, HW, D, T)
    group_ms = {"preprocess": phase_ms["preprocess"], "binning": phase_ms["depth_sort"] + phase_ms["bin"],
                "composite": phase_ms["composite"], "render_bwd": phase_ms["render_bwd"],
                "preprocess_bwd": phase_ms["preprocess_bwd"]}
    dom = max(group_ms, key=group_ms.get)
    peaks = _peaks()
    achieved = pb[dom] / (group_ms[dom] / 1000.0) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 5),
                "peak_source": peaks["source"], "traffic": _traffic(dom, K),
                "algorithmic_bytes_per_launch": pb[dom],
                "note": "algorithmic bytes of the published algorithm for this kernel; the kernel is bound by "
                        "instruction issue, see render_alu"}
    phases = {k: {"ms": round(v, 4), "share": round(v / sum(phase_ms.values()), 4)} for k, v in phase_ms.items()}
    hbm_groups = {k: {"ms": round(v, 4), "algorithmic_bytes": pb[k],
                      "hbm_frac": round(pb[k] / (v / 1000.0) / 1e9 / peaks["hbm_gbs"], 5)} for k, v in group_ms.items()}
    iter_bytes = sum(pb.values())
    E = int(raster.inspect_state(last_state[0], cam.width, cam.height)["n_contrib"].to(torch.int64).sum())
    render_alu = alu_roofline(E, group_ms, pb, peaks)

    plain_gpu = None
    if rank == 0 and not a.no_plain:
        plain_gpu = run_plain_gpu(a, rs, s, target, K, value / world)

    e2e = None
    if not a.no_e2e:
        e2e = run_e2e(a, dgr, sc, rs, dev, barrier, world)

    cpu = None
    if rank == 0 and not a.no_cpu:
        cpu = run_cpu_baseline(sc, a.cpu_budget_s)

    pose_suite = None
    if rank == 0 and not a.no_pose:
        pose_suite = run_pose_suite(a, dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(sc, K, world),
            "render_schedule": {"fwd_batch": sched.fwd_batch, "fwd_warps": sched.fwd_warps,
                                "bwd_batch": sched.bwd_batch},
            "roofline": roofline, "phases": phases, "hbm_by_phase": hbm_groups,
            "iteration_hbm": {"algorithmic_bytes": iter_bytes,
                              "achieved_gbs": round(iter_bytes / (ms_per_step / 1000.0) / 1e9, 2),
                              "frac": round(iter_bytes / (ms_per_step / 1000.0) / 1e9 / peaks["hbm_gbs"], 5)},
            "render_alu": render_alu, "plain_gpu": plain_gpu, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk,
            "gpu_launches": (raster.kernel_launches(sc.camera.width, sc.camera.height)["total"] + 2) * a.steps,
            "pose": pose_suite,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_plain_gpu(a, rs, s, target, K: int, ours_value: float) -> dict:
    """The same iteration on the plain GPU path (cfgs.plain: the published rasteriser's
    structure, 64-bit keys and one radix sort, one thread per pixel, global atomic
    gradients), with the loss as the reference trainer forms it (autograd of the L1 of
    the clamped render, utils/loss_utils.py:15 with scene/gaussian_model_cf.py:885). The
    reference's own CUDA rasteriser is an un-vendored submodule, so this is the GPU
    comparison point for the tuned path on the same device."""
    import torch
    from cfgs import plain

    timers: dict = {}
    cap = [K]  # the instance buffers are sized for the count the last call saw, as upstream keeps its buffers

    def step(tm=None):
        color, radii, depth, alpha, st = plain.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales,
                                                       s.rotations, None, timers=tm, capacity_hint=cap[0])
        cap[0] = st.capacity
        ev = None
        if tm is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        c = color.detach().requires_grad_(True)
        loss = (c.clamp(0.0, 1.0) - target).abs().mean()
        (g,) = torch.autograd.grad(loss, c)
        if ev is not None:
            ev[1].record()
            tm.setdefault("loss", []).append(ev)
        plain.backward(rs, st, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None, g, None, None,
                       timers=tm)
        return st

    for _ in range(max(a.warmup, 1)):
        step()
    torch.cuda.synchronize()
    steps = max(3, a.steps)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(steps):
        st = step(timers)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    phases = {k: round(sum(a_.elapsed_time(b_) for a_, b_ in v) / len(v), 4) for k, v in timers.items()}
    value = 1000.0 / ms
    return {"value": round(value, 4), "unit": UNIT, "ms_per_step": round(ms, 4), "steps": steps,
            "num_rendered": st.num_rendered, "phases_ms": phases,
            "ours_over_plain": round(ours_value / value, 3),
            "what": "reference CUDA rasteriser not available (un-vendored submodule): the build's plain GPU path, "
                    "the published rasteriser's structure (include/cfgs_plain.h), same preprocess and per-Gaussian "
                    "backward kernels, loss by torch autograd as the reference trainer forms it"}


def run_plain(a) -> None:
    """Only the plain GPU path's iteration on the benchmarked workload (for profiling it
    alone); one JSON line."""
    import torch
    import diff_gaussian_rasterization as dgr
    from cfgs import scenes
    dev = torch.device("cuda", 0)
    sc = scenes.scene_large(n=a.n, width=a.width, height=a.height, seed=1)
    cam = sc.camera.to(dev)
    rs = dgr.GaussianRasterizationSettings(cam.height, cam.width, cam.tanfovx, cam.tanfovy, sc.bg.to(dev), 1.0,
                                           cam.viewmatrix, cam.projmatrix, sc.sh_degree, cam.campos, False, False)
    s = sc.to(dev)
    r = run_plain_gpu(a, rs, s, s.target, 1, 1.0)
    r.pop("ours_over_plain")
    line = {"metric": METRIC, "value": r.pop("value"), "unit": UNIT, "n_gpus": 1, "steps": r.pop("steps"),
            "warmup": a.warmup, "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic", "config": {"workload": f"{sc.n} SH{sc.sh_degree} Gaussians, {cam.width}x{cam.height}, "
                                                         "fwd + L1 loss + bwd, plain GPU path"}, **r}
    print(json.dumps(line), flush=True)


def run_e2e(a, dgr, sc, rs, dev, barrier, world) -> dict:
    """Same metric through the public API (GaussianRasterizer + autograd), inputs copied
    from pinned host memory and the loss read back every step. `value`: the inputs of
    step i+1 are copied on a second stream into a second set of device buffers while
    step i computes, and step i's loss is read once step i+1 is enqueued (a training
    loop with host-resident data and asynchronous logging), the median of three timed
    windows; `serial`: each step copies its own inputs first and reads its loss before the
    next begins. Both time every step's copies and its loss read-back."""
    import torch
    from cfgs.loss import l1_loss
    host = {k: getattr(sc, k).pin_memory() for k in ("means3D", "opacities", "shs", "scales", "rotations", "target")}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    raster_mod = dgr.GaussianRasterizer(rs)

    def compute(d):
        means3D = d["means3D"].detach().requires_grad_(True)
        means2D = torch.zeros_like(means3D, requires_grad=True)
        shs = d["shs"].detach().requires_grad_(True)
        opac = d["opacities"].detach().requires_grad_(True)
        scales = d["scales"].detach().requires_grad_(True)
        rots = d["rotations"].detach().requires_grad_(True)
        color, radii, depth, alpha = raster_mod(means3D=means3D, means2D=means2D, opacities=opac, shs=shs,
                                                scales=scales, rotations=rots)
        loss = l1_loss(color, d["target"], clamp=True)
        loss.backward()
        return loss

    def serial_step():
        d = {k: v.to(dev, non_blocking=True) for k, v in host.items()}
        return float(compute(d).item())

    main = torch.cuda.current_stream(dev)
    copy_stream = torch.cuda.Stream(dev)
    bufs = [{k: torch.empty_like(v, device=dev) for k, v in host.items()} for _ in range(2)]
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    freed = [torch.cuda.Event(), torch.cuda.Event()]

    def issue_copy(i):
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(freed[i])
            for k, v in host.items():
                bufs[i][k].copy_(v, non_blocking=True)
            copied[i].record(copy_stream)

    steps = max(3, a.steps)
    loss_host = torch.empty(steps + 2, dtype=torch.float32, pin_memory=True)

    def run_pipelined(n):
        """Step i's loss goes to pinned host memory by an async copy and is read (waiting
        on its event only) once step i+1 is enqueued, so the GPU does not idle while the
        host prepares the next step."""
        for e in freed:
            e.record(main)
        issue_copy(0)
        ready = [torch.cuda.Event() for _ in range(n)]
        for i in range(n):
            cur = i % 2
            main.wait_event(copied[cur])
            issue_copy(1 - cur)  # next step's inputs, behind the step that last used that buffer
            loss = compute(bufs[cur])
            freed[cur].record(main)
            loss_host[i].copy_(loss.detach(), non_blocking=True)
            ready[i].record(main)
            if i > 0:
                ready[i - 1].synchronize()
                float(loss_host[i - 1])
        ready[n - 1].synchronize()
        float(loss_host[n - 1])
        torch.cuda.synchronize()

    for _ in range(max(a.warmup, 1)):
        serial_step()
    run_pipelined(2)
    # the host -> device copies alone (same tensors, same stream), for the breakdown
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        _ = {k: v.to(dev, non_blocking=True) for k, v in host.items()}
    ev1.record()
    torch.cuda.synchronize()
    h2d_ms = ev0.elapsed_time(ev1) / steps

    def timed(fn):
        barrier()
        t0 = time.perf_counter()
        fn()
        barrier()
        return max_over_ranks(time.perf_counter() - t0, world, dev)

    # Host-timed windows of about 60 ms: the collector is paused inside them (a collection
    # pause would land in one window and not another) and the pipelined figure is the
    # median of three windows.
    import gc
    gc.collect()
    gc_was_enabled = gc.isenabled()
    gc.disable()
    try:
        dt_serial = timed(lambda: [serial_step() for _ in range(steps)])
        windows = sorted(timed(lambda: run_pipelined(steps)) for _ in range(3))
    finally:
        if gc_was_enabled:
            gc.enable()
    dt = windows[1]
    return {"value": round(job_rate(world, steps, dt), 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "windows_ms_per_step": [round(w * 1000.0 / steps, 4) for w in windows],
            "d2h_bytes_per_step": 4, "steps": steps, "api": "diff_gaussian_rasterization.GaussianRasterizer",
            "copies": "next step's inputs on a second stream during the current step",
            "loss_read": "every step's loss copied to pinned host memory and read after the next step is enqueued",
            "ms_per_step": round(dt * 1000.0 / steps, 4),
            "serial": {"value": round(job_rate(world, steps, dt_serial), 4), "ms_per_step": round(dt_serial * 1000.0 / steps, 4)},
            "h2d_ms_alone": round(h2d_ms, 4), "h2d_gb_per_s": round(h2d / (h2d_ms / 1000.0) / 1e9, 1)}


# ---------------------------------------------------------------------------
# CPU oracle: the reported CPU baseline and the --impl reference arm
# ---------------------------------------------------------------------------
def _oracle_iteration(sc, Oracle):
    import numpy as np
    o = Oracle.from_scene(sc).forward()
    c = o.color
    diff = np.clip(c, 0, 1) - sc.target.numpy()
    g = (np.sign(diff) * ((c >= 0) & (c <= 1))).astype(np.float32) / c.size
    o.backward(g)
    return o.K


def run_cpu_baseline(sc, budget_s: float) -> dict:
    from oracle import c_oracle
    cores = _cores()
    c_oracle.set_threads(cores)
    times = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        _oracle_iteration(sc, c_oracle.Oracle)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start + times[-1] > budget_s or len(times) >= 5:
            break
    t = statistics.median(times)
    return {"value": round(1.0 / t, 5), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(times)} full fwd+bwd iteration(s) of the same workload, median {t:.2f} s"}


def run_reference(a) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from cfgs import scenes
    from oracle import c_oracle
    cores = _cores()
    c_oracle.set_threads(cores)
    sc = scenes.scene_large(n=a.n, width=a.width, height=a.height, seed=1)
    t_w, K = 0.0, 0
    for _ in range(max(a.warmup, 1)):
        t0 = time.perf_counter()
        K = _oracle_iteration(sc, c_oracle.Oracle)
        t_w = time.perf_counter() - t0
    # a rate: when the requested steps would run past ~150 s, time fewer of them
    steps = max(1, min(a.steps, int(150.0 / max(t_w, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(steps):
        _oracle_iteration(sc, c_oracle.Oracle)
    dt = time.perf_counter() - t0
    value = steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1000 * dt / steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(sc, K, int(os.environ.get("WORLD_SIZE", "1"))),
        "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step one full fwd+bwd iteration ({steps} of {a.steps} steps timed)"},
        "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference rasteriser is CUDA-only and its source is not in the reference tree; this arm "
                "times the CPU restatement of its algorithm (oracle port) on all host cores",
    }
    print(json.dumps(line), flush=True)


def _pose_setup(dev, count, seed=3):
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import pose, scenes
    specs = scenes.batch_specs(count, seed=seed)
    probs, cams = [], []
    for (w, h, n, sd) in specs:
        sc = scenes.scene_pose(width=w, height=h, n=n, seed=sd)
        probs.append(pose.make_problem(sc, dev))
        cams.append(sc.camera)
    return specs, probs, cams


def _pct(x, q):
    import numpy as np
    return round(float(np.percentile(np.asarray(x, np.float64), q)), 4)


def pose_single(dev, engine_reps: int = 5, plain_reps: int = 2) -> dict:
    """One CF-3DGS relative-pose solve (640x360, one Gaussian per pixel, 300 Adam
    iterations, lr 1e-3, RGB L1; trainer/cf3dgs_trainer.py:261-285), end to end per
    solve: the plain path (PyTorch pose algebra + autograd + torch Adam around the
    rasteriser: the reference's structure), the fused pose kernels behind autograd, and
    the solve engine (batched kernels, CUDA-graph replays, no host synchronisation inside
    the 300 iterations; its setup inside the timed region)."""
    import torch
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import autotune, batch, pose, scenes
    prob = pose.make_problem(scenes.scene_pose(width=640, height=360, seed=2), dev)
    res = {}
    for mode, reps in (("plain", plain_reps), ("fused", plain_reps)):
        pose.time_solves(prob, mode, count=1)
        sps, lat = pose.time_solves(prob, mode, count=reps)
        xi, _ = pose.solve(prob, mode=mode)
        res[mode] = {"solves_per_s": sps, "latency_s": lat, "xi": xi}
    tuner = autotune.Autotuner()

    def engine_solve():
        return batch.BatchSolver([prob], autotune=tuner).solve(300).xi[0]

    engine_solve()
    lat = []
    for _ in range(engine_reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xi = engine_solve()
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t0)
    dang, dtr = pose.pose_error(res["plain"]["xi"], res["fused"]["xi"])
    eang, etr = pose.pose_error(res["plain"]["xi"], xi)
    gerr = pose.pose_error(xi, prob.xi_gt)
    sps = len(lat) / sum(lat)
    return {"workload": "CF-3DGS relative pose solve, 230400 SH0 Gaussians, 640x360, 300 Adam iterations, RGB L1",
            "solves_per_s": round(sps, 4), "latency_p50_s": _pct(lat, 50), "latency_p99_s": _pct(lat, 99),
            "solves_timed": len(lat),
            "plain_solves_per_s": round(res["plain"]["solves_per_s"], 4),
            "plain_latency_p50_s": _pct(res["plain"]["latency_s"], 50),
            "plain_latency_p99_s": _pct(res["plain"]["latency_s"], 99),
            "fused_autograd_solves_per_s": round(res["fused"]["solves_per_s"], 4),
            "speedup_vs_plain": round(sps / res["plain"]["solves_per_s"], 3),
            "plain_vs_fused": {"rot_deg": dang, "trans": dtr},
            "plain_vs_engine": {"rot_deg": eang, "trans": etr},
            "engine_vs_ground_truth": {"rot_deg": gerr[0], "trans": gerr[1]},
            "path": "solve engine (cfgs_batch_iteration in CUDA graphs), setup included",
            "render_schedule": str(autotune.get_schedule())}


def run_pose(a) -> None:
    import torch
    dev = torch.device("cuda", 0)
    r = pose_single(dev, engine_reps=max(3, a.steps // 2), plain_reps=max(2, a.steps // 5))
    line = {"metric": "pose solves/s (640x360, 300 iterations)", "value": r["solves_per_s"], "unit": "solves/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"], "path": r["path"]}, **r}
    print(json.dumps(line), flush=True)


def run_pose_iter(a) -> None:
    """One iteration of the solve engine on the 640x360 pose problem, eager launches (no
    graph): W untimed iterations, then K timed with CUDA events; a small, fixed sequence
    of launches for profilers."""
    import torch
    import diff_gaussian_rasterization  # noqa: F401
    from cfgs import batch, pose, scenes
    dev = torch.device("cuda", 0)
    prob = pose.make_problem(scenes.scene_pose(width=640, height=360, seed=2), dev)
    bs = batch.BatchSolver([prob])
    from cfgs import autotune
    autotune.set_schedule(autotune.Schedule(bin_launch=a.bin_launch))
    args = bs.prepare()
    K0 = bs.capacity
    for _ in range(a.warmup):
        bs.iterate(args)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record()
    for _ in range(a.steps):
        bs.iterate(args)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / max(a.steps, 1)
    print(json.dumps({"metric": "pose-solve engine iteration (640x360, eager launches)", "value": round(ms, 4),
                      "unit": "ms/iteration", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
                      "higher_is_better": False, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "CF-3DGS relative pose solve, 230400 SH0 Gaussians, 640x360",
                                 "instance_capacity": int(K0), "bin_launch": a.bin_launch}}), flush=True)


def run_batch_iter(a) -> None:
    """One iteration of the solve engine on the 64-solve mix, eager launches (no graph):
    W untimed iterations, then K timed with CUDA events; for profilers."""
    import torch
    from cfgs import batch
    dev = torch.device("cuda", 0)
    _, probs, _ = _pose_setup(dev, 64)
    bs = batch.BatchSolver(probs)
    from cfgs import autotune
    autotune.set_schedule(autotune.Schedule(bin_launch=a.bin_launch))
    args = bs.prepare()
    for _ in range(a.warmup):
        bs.iterate(args)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("batch_iter")  # lets a profiler take the timed iterations alone
    t0.record()
    for _ in range(a.steps):
        bs.iterate(args)
    t1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = t0.elapsed_time(t1) / max(a.steps, 1)
    print(json.dumps({"metric": "pose-solve engine iteration (64 uneven solves, eager launches)",
                      "value": round(ms, 4), "unit": "ms/iteration", "n_gpus": 1, "steps": a.steps,
                      "warmup": a.warmup, "higher_is_better": False, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "64 CF-3DGS pose solves, N log-uniform [5e4,5e5], "
                                             "320x180/640x360/960x540",
                                 "instance_capacity": int(bs.capacity), "bin_launch": a.bin_launch}}),
          flush=True)


def pose_batch(dev, probs, sample: int = 8) -> dict:
    """64 pose solves (N log-uniform in [5e4, 5e5], resolutions 320x180/640x360/960x540)
    batched (one launch per stage, CUDA-graph replays) vs the same solves one after
    another on the plain path, timed on the first `sample` of them."""
    import numpy as np
    from cfgs import batch, pose
    bs = batch.BatchSolver(probs, autotune=True)
    bs.solve(300)  # tunes the render schedule for this batch shape (cached), untimed
    r = bs.solve(300)
    batch.solve_sequential(probs[:1], 300, "plain")
    xs, lat = batch.solve_sequential(probs[:sample], 300, "plain")
    plain_sps = sample / sum(lat)
    xf, latf = batch.solve_sequential(probs[:sample], 300, "fused")
    agree = [pose.pose_error(xs[i], r.xi[i]) for i in range(sample)]
    sps = len(probs) / r.seconds
    return {"workload": f"{len(probs)} CF-3DGS pose solves, N log-uniform [5e4,5e5], 320x180/640x360/960x540, "
                        "300 Adam iterations each",
            "solves_per_s": round(sps, 4), "batch_seconds": round(r.seconds, 3),
            "latency_s": round(r.seconds, 3),
            "ms_per_iteration": round(1000 * r.seconds / 300, 3),
            "total_gaussians": int(sum(p.xyz.shape[0] for p in probs)), "num_rendered": r.num_rendered0,
            "plain_sequential_solves_per_s": round(plain_sps, 4), "plain_sample": sample,
            "plain_latency_p50_s": _pct(lat, 50), "plain_latency_p99_s": _pct(lat, 99),
            "fused_sequential_solves_per_s": round(sample / sum(latf), 4),
            "speedup_vs_plain": round(sps / plain_sps, 3),
            "batched_vs_fused_single_bit_identical": bool(np.array_equal(np.float32(xf), np.float32(r.xi[:sample]))),
            "batched_vs_plain_max": {"rot_deg": max(x[0] for x in agree), "trans": max(x[1] for x in agree)},
            "graph_chunk": bs.graph_chunk, "render_schedule": str(bs.schedule)}


def run_batch(a) -> None:
    import torch
    dev = torch.device("cuda", 0)
    _, probs, _ = _pose_setup(dev, 64)
    r = pose_batch(dev, probs, sample=max(2, min(8, a.steps)))
    line = {"metric": "batched pose solves/s (64 uneven solves)", "value": r["solves_per_s"], "unit": "solves/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"]}, **r}
    print(json.dumps(line), flush=True)


def pose_serve(dev, payloads, target, rate: float, seconds: float, plain_seconds: float, slots: int = 64,
               seed: int = 11) -> dict:
    """A Poisson stream of `rate` req/s (90% pose solves of the 64-solve mix, 10% renders
    of a device-resident 1M-Gaussian SH3 scene at 1920x1080) served by the
    continuous-batching server for `seconds` and by the plain FIFO loop for
    `plain_seconds` (requests still queued or running at the end are not counted)."""
    from cfgs import serve
    out = {}
    for name, secs in (("continuous", seconds), ("plain_fifo", plain_seconds)):
        stream = serve.poisson_stream(rate, secs, 0.9, len(payloads), 1, seed=seed)
        if name == "continuous":
            srv = serve.ContinuousBatchServer(payloads, [target], dev, max_slots=slots, hbm_budget=150e9)
        else:
            srv = serve.PlainFifoServer(payloads, [target], dev)
        st = srv.run(stream, wall_limit=secs)
        s = st.summary(name)
        s["arrived"] = len(stream)
        s["stream_seconds"] = secs
        out[name] = s
    c, p = out["continuous"], out["plain_fifo"]
    return {"workload": f"Poisson {rate:g} req/s, 90% pose solves (64-solve mix), 10% renders of 1M SH3 Gaussians "
                        "at 1920x1080", "hbm_budget_gb": 150, "max_slots": slots, "epoch_iterations": 25,
            "continuous": c, "plain_fifo": p,
            "pose_throughput_speedup_vs_plain": round(c["pose_solves_per_s"] / max(p["pose_solves_per_s"], 1e-9), 3)}


def run_serve(a) -> None:
    import torch
    from cfgs import scenes, serve
    dev = torch.device("cuda", 0)
    _, probs, cams = _pose_setup(dev, 64)
    payloads = [serve.payload_from_problem(p, c) for p, c in zip(probs, cams)]
    del probs
    target = serve.RenderTarget(scenes.scene_large(), dev)
    target.render()
    torch.cuda.synchronize()
    r = pose_serve(dev, payloads, target, a.serve_rate, a.serve_seconds, a.serve_seconds, a.serve_slots)
    line = {"metric": "served requests/s (90% pose solves, 10% 1080p renders)",
            "value": r["continuous"]["throughput_req_s"], "unit": "req/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic", "config": {"workload": r["workload"]}, **r}
    print(json.dumps(line), flush=True)


def run_pose_suite(a, dev) -> dict:
    """The metric's second half, measured in the default run: solves/s and latency of
    the pose-solve workloads against the plain path, with the clocks of their timed
    regions. One 640x360 solve; the 64-solve batch (plain timed on 8 of them); the served
    stream at 200 req/s (continuous server for 60 s, plain FIFO for 20 s: both are
    saturated, so the shorter window gives the plain loop's rate) and at a rate the
    continuous server sustains (8 req/s, 20 s each), for latencies without a standing
    queue."""
    import torch
    from cfgs import scenes, serve
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    out = {"single": pose_single(dev)}
    _, probs, cams = _pose_setup(dev, 64)
    out["batch64"] = pose_batch(dev, probs, sample=8)
    payloads = [serve.payload_from_problem(p, c) for p, c in zip(probs, cams)]
    del probs
    torch.cuda.empty_cache()
    target = serve.RenderTarget(scenes.scene_large(), dev)
    target.render()
    torch.cuda.synchronize()
    out["served_200"] = pose_serve(dev, payloads, target, a.serve_rate, a.serve_seconds, min(20.0, a.serve_seconds),
                                   a.serve_slots)
    out["served_sustained"] = pose_serve(dev, payloads, target, 8.0, 20.0, 20.0, a.serve_slots, seed=12)
    out["clocks"] = clocks.stop()
    return out


def run_ssim(a) -> None:
    """SSIM loss (the pose loss's 0.2 (1 - SSIM) term, utils/loss_utils.py:33-58) on a
    3x1080x1920 image pair, forward + backward per step: the fused kernels vs the
    reference's formulation in PyTorch (depthwise conv2d + autograd) on the same GPU."""
    import torch
    import torch.nn.functional as F
    from cfgs import ssim as ssim_mod
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(0)
    C, H, W = 3, 1080, 1920
    x0 = torch.rand(C, H, W, generator=g).to(dev)
    y = (x0 + 0.1 * torch.randn(C, H, W, generator=g).to(dev)).clamp(0, 1)
    w1 = torch.exp(-((torch.arange(11, dtype=torch.float64) - 5) ** 2) / (2 * 1.5 ** 2))
    w1 = (w1 / w1.sum()).float()
    win = (w1[:, None] @ w1[None, :]).expand(C, 1, 11, 11).contiguous().to(dev)

    def torch_ssim(x):
        xb, yb = x[None], y[None]
        mu1, mu2 = F.conv2d(xb, win, padding=5, groups=C), F.conv2d(yb, win, padding=5, groups=C)
        s11 = F.conv2d(xb * xb, win, padding=5, groups=C) - mu1 * mu1
        s22 = F.conv2d(yb * yb, win, padding=5, groups=C) - mu2 * mu2
        s12 = F.conv2d(xb * yb, win, padding=5, groups=C) - mu1 * mu2
        m = ((2 * mu1 * mu2 + 1e-4) * (2 * s12 + 9e-4)) / ((mu1 * mu1 + mu2 * mu2 + 1e-4) * (s11 + s22 + 9e-4))
        return m.mean()

    def timed(fn, steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(a.warmup):
            fn()
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(steps):
            fn()
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / steps

    def step(f):
        x = x0.clone().requires_grad_(True)
        (0.2 * (1.0 - f(x))).backward()
        return x.grad

    def fused_ssim(x):
        return ssim_mod.ssim(x, y)

    from cfgs import native
    lib = native.load()
    scratch = torch.empty(int(lib.cfgs_ssim_scratch_bytes(C, H, W)), dtype=torch.uint8, device=dev)
    mean = torch.empty((), device=dev)
    gscale = torch.full((), -0.2, device=dev)
    dx = torch.empty_like(x0)
    st = torch.cuda.current_stream(dev).cuda_stream

    def kernels_only():
        native.check(lib.cfgs_ssim_forward(C, H, W, x0.data_ptr(), y.data_ptr(), scratch.data_ptr(),
                                           mean.data_ptr(), st), "cfgs_ssim_forward")
        native.check(lib.cfgs_ssim_backward(C, H, W, x0.data_ptr(), y.data_ptr(), scratch.data_ptr(),
                                            gscale.data_ptr(), dx.data_ptr(), st), "cfgs_ssim_backward")

    ms_kernels = timed(kernels_only, a.steps)
    ms_fused = timed(lambda: step(fused_ssim), a.steps)
    ms_torch = timed(lambda: step(torch_ssim), max(3, a.steps // 4))
    gf, gt = step(fused_ssim), step(torch_ssim)
    rel = float((gf - gt).abs().max() / gt.abs().max())
    vf, vt = float(ssim_mod.ssim(x0, y)), float(torch_ssim(x0))
    n = C * H * W
    algo = 4 * n * (2 + 3 + 3 + 2 + 1)  # fwd: read 2 images, write 3 maps; bwd: read 3 maps + 2 images, write 1
    peaks = _peaks()
    achieved = algo / (ms_kernels / 1000.0) / 1e9
    line = {"metric": "SSIM loss fwd+bwd per s (3x1080x1920)", "value": round(1000.0 / ms_kernels, 3),
            "unit": "steps/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "0.2 (1 - SSIM) of a 3x1080x1920 image pair, 11x11 window, fwd + bwd",
                       "value": "the two C-ABI calls on device buffers",
                       "step": "autograd step through cfgs.ssim.ssim (clone, loss, backward)"},
            "ms_per_step": round(ms_kernels, 4), "autograd_ms_per_step": round(ms_fused, 4),
            "torch_ms_per_step": round(ms_torch, 4),
            "speedup_vs_torch": round(ms_torch / ms_fused, 3),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": round(achieved / peaks["hbm_gbs"], 5), "algorithmic_bytes": algo},
            "ssim_fused": vf, "ssim_torch": vt, "grad_max_rel_diff_vs_torch": rel}
    print(json.dumps(line), flush=True)


def run_init(a) -> None:
    """Local-Gaussian initialisation of one frame (the steps before each pose solve):
    640x360 depth -> points -> 0.01 voxel down-sampling -> three-nearest-neighbour
    scales -> initial Gaussians, and the kNN step alone on 1,000,000 points. CPU
    comparison on the host cores: the C restatement of the voxel step and scipy's
    k-d tree for the neighbours."""
    import time
    import numpy as np
    import torch
    from cfgs import pointcloud
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(0)
    v, u = np.mgrid[0:360, 0:640].astype(np.float32)
    depth = (2.0 + 0.5 * np.sin(u / 37.0) + 0.3 * np.cos(v / 23.0) + 0.02 * rng.standard_normal((360, 640)))
    depth = depth.astype(np.float32)
    rgb = rng.uniform(0, 1, (360 * 640, 3)).astype(np.float32)
    K = np.array([[500.0, 0, 320.0], [0, 500.0, 180.0], [0, 0, 1]])
    d_dev, rgb_dev = torch.tensor(depth, device=dev), torch.tensor(rgb, device=dev)

    def frame():
        pts = pointcloud.depth_to_points(d_dev, K)
        p, c = pointcloud.voxel_down_sample(pts, rgb_dev, 0.01)
        return pointcloud.gaussians_from_points(p, c)

    for _ in range(a.warmup):
        g = frame()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        g = frame()
    torch.cuda.synchronize()
    ms_frame = (time.perf_counter() - t0) * 1000.0 / a.steps
    n_vox = int(g["xyz"].shape[0])
    big = torch.randn(1_000_000, 3, device=dev)
    for _ in range(a.warmup):
        pointcloud.dist_cuda2(big)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(a.steps):
        pointcloud.dist_cuda2(big)
    ev1.record()
    torch.cuda.synchronize()
    ms_knn = ev0.elapsed_time(ev1) / a.steps
    cpu = {}
    if not a.no_cpu:
        from oracle import c_oracle
        pts_h = pointcloud.depth_to_points(d_dev, K).cpu().numpy()
        t0 = time.perf_counter()
        vp, vc = c_oracle.voxel_down_sample(pts_h, rgb, 0.01)
        cpu["voxel_ms_c_1thread"] = round((time.perf_counter() - t0) * 1000.0, 2)
        try:
            from scipy.spatial import cKDTree
            t0 = time.perf_counter()
            cKDTree(vp.astype(np.float64)).query(vp.astype(np.float64), k=4, workers=-1)
            cpu["knn_frame_ms_scipy"] = round((time.perf_counter() - t0) * 1000.0, 2)
            bh = big.cpu().numpy().astype(np.float64)
            t0 = time.perf_counter()
            cKDTree(bh).query(bh, k=4, workers=-1)
            cpu["knn_1M_ms_scipy"] = round((time.perf_counter() - t0) * 1000.0, 2)
        except ImportError:
            pass
        cpu["cores"] = len(os.sched_getaffinity(0))
    line = {"metric": "frame initialisations/s (640x360 depth -> local Gaussians)", "value": round(1000.0 / ms_frame, 3),
            "unit": "frames/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "depth_to_points + voxel_down_sample(0.01) + distCUDA2 scales + create_from_pcd, "
                                   "640x360", "points": 640 * 360, "voxels": n_vox},
            "ms_per_frame": round(ms_frame, 4), "knn_1M_points_ms": round(ms_knn, 4), "cpu": cpu}
    print(json.dumps(line), flush=True)


def run_optim(a) -> None:
    """Gaussian-parameter optimisation of a 1,000,000-Gaussian SH3 model: the Adam step
    over the six parameter groups (fused, one launch) vs torch.optim.Adam (multi-tensor),
    and densify_and_prune vs the reference's PyTorch functions on the GPU."""
    import torch
    from cfgs import densify
    from oracle import densify_oracle
    dev = torch.device("cuda", 0)
    n = 1_000_000
    g = torch.Generator(device="cpu").manual_seed(0)
    p0 = {"xyz": torch.randn(n, 3, generator=g), "f_dc": torch.randn(n, 1, 3, generator=g),
          "f_rest": 0.1 * torch.randn(n, 15, 3, generator=g), "opacity": 2.0 * torch.randn(n, 1, generator=g),
          "scaling": torch.randn(n, 3, generator=g) - 4.0, "rotation": torch.randn(n, 4, generator=g)}
    p0 = {k: v.to(dev) for k, v in p0.items()}
    lrs = {"xyz": 5e-4, "f_dc": 2.5e-3, "f_rest": 1.25e-4, "opacity": 0.05, "scaling": 5e-3, "rotation": 1e-3}
    grads = {k: 0.01 * torch.randn_like(v) for k, v in p0.items()}
    opt = densify.GaussianOptimizer(p0, lrs)
    ref = {k: torch.nn.Parameter(v.clone()) for k, v in p0.items()}
    for k in ref:
        ref[k].grad = grads[k]
    topt = torch.optim.Adam([{"params": [ref[k]], "lr": lrs[k]} for k in densify.GROUPS], lr=0.0, eps=1e-15)

    def timed(fn, steps):
        for _ in range(a.warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_adam = timed(lambda: opt.step(grads), a.steps)
    ms_torch = timed(topt.step, a.steps)
    elems = sum(v.numel() for v in p0.values())
    algo = 28 * elems  # read p, g, m, v; write p, m, v (float32)
    peaks = _peaks()
    achieved = algo / (ms_adam / 1000.0) / 1e9
    # densify_and_prune on the same statistics and draws
    accum = torch.where(torch.rand(n, device=dev) < 0.2, 5e-4, 1e-5)
    denom = torch.ones(n, device=dev)
    kw = dict(max_grad=2e-4, min_opacity=0.005, extent=3.0, max_screen_size=20, percent_dense=0.01)

    pool = []

    def prepare(count):
        pool.clear()
        for _ in range(count):
            o = densify.GaussianOptimizer(p0, lrs)
            o.grad_accum.copy_(accum)
            o.denom.copy_(denom)
            pool.append(o)

    def ours():
        return pool.pop().densify_and_prune(z=zz, **kw)

    sel = ((accum / denom) >= 2e-4) & (p0["scaling"].exp().max(1).values > 0.03)
    zz = torch.randn(2, int(sel.sum()), 3, device=dev)
    zeros = {k: torch.zeros_like(v) for k, v in p0.items()}

    def theirs():
        return densify_oracle.densify_and_prune(p0, zeros, zeros, accum, denom, z=zz, **kw)

    dens_steps = max(3, a.steps // 4)
    prepare(a.warmup + dens_steps)  # fresh optimiser states, built outside the timed region
    ms_dens = timed(ours, dens_steps)
    ms_dens_torch = timed(theirs, dens_steps)
    prepare(1)
    res = ours()
    pool.clear()
    line = {"metric": "Gaussian Adam steps/s (1M SH3 Gaussians, 6 groups)", "value": round(1000.0 / ms_adam, 3),
            "unit": "steps/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "Adam over xyz, f_dc, f_rest, opacity, scaling, rotation of 1,000,000 SH3 Gaussians",
                       "elements": elems},
            "ms_per_step": round(ms_adam, 4), "torch_adam_ms": round(ms_torch, 4),
            "speedup_vs_torch_adam": round(ms_torch / ms_adam, 3),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": round(achieved / peaks["hbm_gbs"], 5), "algorithmic_bytes": algo},
            "densify_and_prune_ms": round(ms_dens, 3), "torch_densify_and_prune_ms": round(ms_dens_torch, 3),
            "densify_counts": res}
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "plain":
        run_plain(a)
    elif a.workload == "pose":
        run_pose(a)
    elif a.workload == "pose_iter":
        run_pose_iter(a)
    elif a.workload == "batch":
        run_batch(a)
    elif a.workload == "batch_iter":
        run_batch_iter(a)
    elif a.workload == "serve":
        run_serve(a)
    elif a.workload == "ssim":
        run_ssim(a)
    elif a.workload == "init":
        run_init(a)
    elif a.workload == "optim":
        run_optim(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
