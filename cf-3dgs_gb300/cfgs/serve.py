"""Serving pose-solve and render requests on one GPU with continuous batching.

Requests arrive over time (a Poisson stream in the benchmark). Pose-solve requests
carry the local Gaussians of a frame, the camera and the next frame (the CF-3DGS
relative-pose solve, trainer/cf3dgs_trainer.py:261-285); render requests ask for a
1920x1080 view of a registered 1M-Gaussian scene that stays on the device.

ContinuousBatchServer runs in epochs of `epoch` Adam iterations. At every epoch
boundary it retires the solves that reached their iteration count, admits queued
pose requests in arrival order as slots and the HBM budget allow (their Gaussians and
optimiser state are uploaded once and stay on the device), repacks the active solves
into one batch (cfgs.batch) and runs the epoch; render requests run on a second CUDA
stream as they arrive, overlapping the solve epochs. A solve's arithmetic depends only
on its own data, so its result is the same alone and in any mix.

PlainFifoServer is the comparison: one request at a time in arrival order, pose
solves on the plain path (PyTorch SE(3) + autograd + torch.optim.Adam, the reference's
structure) and renders through the drop-in forward.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import batch as batch_mod
from . import pose as pose_mod


@dataclass
class Request:
    rid: int
    kind: str            # "pose" | "render"
    arrival: float       # seconds after the stream starts
    payload: int         # index into the server's payload lists
    start: float = math.nan
    done: float = math.nan
    result: object = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_stream(rate: float, duration: float, pose_frac: float, n_pose: int, n_render: int,
                   seed: int = 0) -> list[Request]:
    """Arrivals of a Poisson process of `rate` req/s over `duration` s; each request is a
    pose solve with probability pose_frac (payload drawn uniformly), else a render."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        if rng.uniform() < pose_frac:
            out.append(Request(len(out), "pose", t, int(rng.integers(0, n_pose))))
        else:
            out.append(Request(len(out), "render", t, int(rng.integers(0, max(n_render, 1)))))


@dataclass
class PosePayload:
    """A pose request as a client sends it: host (pinned) tensors."""
    xyz: torch.Tensor
    opacities: torch.Tensor
    shs: torch.Tensor
    scales: torch.Tensor
    rotations: torch.Tensor
    target: torch.Tensor
    camera: object        # cfgs.scenes.Camera (host)
    sh_degree: int

    @property
    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in (self.xyz, self.opacities, self.shs, self.scales,
                                                            self.rotations, self.target))


def payload_from_problem(prob: pose_mod.PoseProblem, camera) -> PosePayload:
    pin = lambda t: t.detach().cpu().contiguous().pin_memory()
    return PosePayload(pin(prob.xyz), pin(prob.opacities), pin(prob.shs), pin(prob.scales), pin(prob.rotations),
                       pin(prob.target), camera, prob.sh_degree)


def upload(payload: PosePayload, device) -> pose_mod.PoseProblem:
    """Device copy of a pose request (the H2D part of its latency)."""
    import diff_gaussian_rasterization as dgr
    d = lambda t: t.to(device, non_blocking=True)
    cam = payload.camera.to(device)
    bg = torch.zeros(3, device=device)
    rs = dgr.GaussianRasterizationSettings(cam.height, cam.width, cam.tanfovx, cam.tanfovy, bg, 1.0, cam.viewmatrix,
                                           cam.projmatrix, payload.sh_degree, cam.campos, False, False)
    return pose_mod.PoseProblem(d(payload.xyz), d(payload.opacities), d(payload.shs), d(payload.scales),
                                d(payload.rotations), payload.sh_degree, rs, d(payload.target))


class RenderTarget:
    """A device-resident scene rendered on request (forward only)."""

    def __init__(self, scene, device):
        import diff_gaussian_rasterization as dgr
        s = scene.to(device)
        cam = s.camera
        self.rs = dgr.GaussianRasterizationSettings(cam.height, cam.width, cam.tanfovx, cam.tanfovy, s.bg, 1.0,
                                                    cam.viewmatrix, cam.projmatrix, s.sh_degree, cam.campos,
                                                    False, False)
        self.s = s
        self.m2 = torch.zeros_like(s.means3D)
        self.rast = dgr.GaussianRasterizer(self.rs)

    def render(self) -> torch.Tensor:
        with torch.no_grad():
            color, _, _, _ = self.rast(means3D=self.s.means3D, means2D=self.m2, opacities=self.s.opacities,
                                       shs=self.s.shs, scales=self.s.scales, rotations=self.s.rotations)
        return color


def solve_bytes(payload: PosePayload) -> int:
    """Device memory a solve holds while active: its inputs and target, its share of the
    per-Gaussian workspace and of the per-instance workspaces (about 2 tile instances
    per Gaussian for these scenes, 28 + 48 bytes each), and its render."""
    n = payload.xyz.shape[0]
    px = payload.target.numel() // 3
    return payload.nbytes + n * 64 + n * 2 * 76 + px * 3 * 4 * 2 + px * 8


@dataclass
class ServeStats:
    completed: list = field(default_factory=list)
    wall: float = 0.0
    admitted_peak: int = 0
    epochs: int = 0

    def summary(self, name: str) -> dict:
        lat = np.array([r.latency for r in self.completed]) if self.completed else np.array([math.nan])
        kinds = {k: [r for r in self.completed if r.kind == k] for k in ("pose", "render")}
        pl = np.array([r.latency for r in kinds["pose"]]) if kinds["pose"] else np.array([math.nan])
        return {"server": name, "completed": len(self.completed), "wall_s": round(self.wall, 3),
                "throughput_req_s": round(len(self.completed) / self.wall, 4) if self.wall else None,
                "pose_solves_per_s": round(len(kinds["pose"]) / self.wall, 4) if self.wall else None,
                "renders_per_s": round(len(kinds["render"]) / self.wall, 4) if self.wall else None,
                "latency_p50_s": round(float(np.nanpercentile(lat, 50)), 4),
                "latency_p99_s": round(float(np.nanpercentile(lat, 99)), 4),
                "pose_latency_p50_s": round(float(np.nanpercentile(pl, 50)), 4),
                "pose_latency_p99_s": round(float(np.nanpercentile(pl, 99)), 4),
                "peak_active_solves": self.admitted_peak, "epochs": self.epochs}


class ContinuousBatchServer:
    def __init__(self, pose_payloads: list[PosePayload], render_targets: list[RenderTarget], device="cuda",
                 max_slots: int = 64, hbm_budget: float = 150e9, epoch: int = 25, iters: int = 300,
                 use_graph: bool = True):
        self.pose_payloads = pose_payloads
        self.render_targets = render_targets
        self.dev = torch.device(device)
        self.max_slots, self.hbm_budget, self.epoch, self.iters = max_slots, hbm_budget, epoch, iters
        self.use_graph = use_graph
        if iters % epoch:
            raise ValueError("iters must be a multiple of epoch")

    def run(self, stream: list[Request], wall_limit: float = math.inf, stop_admitting_after: float = math.inf):
        """Serves `stream` (sorted by arrival) in real time from now. Stops when every
        request is done, or at wall_limit (requests still queued or active then are
        not counted)."""
        stats = ServeStats()
        pending = deque(stream)
        queue: deque = deque()
        active: list[dict] = []      # {"req", "prob", "xi", "adam", "it", "bytes"}
        renders: list[tuple] = []    # (req, event, host image)
        rstream = torch.cuda.Stream(self.dev)
        pool: list[torch.Tensor] = []
        used = 0
        bs, members, epoch_ev, retries = None, None, None, 0
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0

        def poll_renders():
            keep = []
            for req, ev, host in renders:
                if ev.query():
                    req.done = clock()
                    req.result = float(host.double().sum())  # the image reached the host
                    pool.append(host)
                    stats.completed.append(req)
                else:
                    keep.append((req, ev, host))
            renders[:] = keep

        def ingest():
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                if r.kind != "render":
                    queue.append(r)
                    continue
                r.start = clock()
                with torch.cuda.stream(rstream):
                    img = self.render_targets[r.payload].render()
                    host = pool.pop() if pool else torch.empty(img.shape, dtype=img.dtype, pin_memory=True)
                    host.copy_(img, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(rstream)
                renders.append((r, ev, host))

        while True:
            if clock() > wall_limit:
                break
            ingest()
            poll_renders()
            if epoch_ev is not None:                   # an epoch is on the GPU
                if not epoch_ev.query():
                    time.sleep(0.0002)
                    continue
                epoch_ev = None
                if not bs.finish():                    # capacity outgrown: rerun the epoch
                    retries += 1
                    if retries > 3:
                        raise RuntimeError("tile-instance capacity kept overflowing")
                    epoch_ev = bs.launch(self.epoch)
                    continue
                retries = 0
                stats.epochs += 1
                retired = []
                for s, a in enumerate(active):
                    a["it"] += self.epoch
                    if a["it"] >= self.iters:
                        a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
                        a["req"].result = a["xi"].double().cpu().numpy()
                        a["req"].done = clock()
                        stats.completed.append(a["req"])
                        retired.append(s)
                if retired:
                    for s, a in enumerate(active):     # keep the survivors' optimiser state
                        a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
                    for s in reversed(retired):
                        used -= active[s]["bytes"]
                        del active[s]
            # epoch boundary: admission in arrival order, within slots and the HBM budget
            admitted = False
            while queue and len(active) < self.max_slots and clock() <= stop_admitting_after:
                r = queue[0]
                pl = self.pose_payloads[r.payload]
                need = solve_bytes(pl)
                if used + need > self.hbm_budget and active:
                    break
                queue.popleft()
                r.start = clock()
                if bs is not None and members == [id(a["req"]) for a in active]:
                    for s, a in enumerate(active):     # leaving the old batch: save its state
                        a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
                active.append({"req": r, "prob": upload(pl, self.dev), "xi": torch.zeros(6, device=self.dev),
                               "adam": torch.zeros(16, device=self.dev), "it": 0, "bytes": need})
                used += need
                admitted = True
            stats.admitted_peak = max(stats.admitted_peak, len(active))
            if not active:
                if not pending and not queue and not renders:
                    break
                time.sleep(0.0005)
                continue
            ids = [id(a["req"]) for a in active]
            if bs is None or admitted or ids != members:  # membership changed: repack
                bs = batch_mod.BatchSolver([a["prob"] for a in active], use_graph=self.use_graph,
                                           graph_chunk=self.epoch)
                bs.load_state(torch.stack([a["xi"] for a in active]), torch.stack([a["adam"] for a in active]))
                members = ids
            epoch_ev = bs.launch(self.epoch)
        rstream.synchronize()
        poll_renders()
        stats.wall = clock()
        return stats


class PlainFifoServer:
    """One request at a time, in arrival order, on the plain single-solve path."""

    def __init__(self, pose_payloads, render_targets, device="cuda", iters: int = 300, mode: str = "plain"):
        self.pose_payloads, self.render_targets = pose_payloads, render_targets
        self.dev = torch.device(device)
        self.iters, self.mode = iters, mode

    def run(self, stream: list[Request], wall_limit: float = math.inf):
        stats = ServeStats()
        pending = deque(stream)
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0
        while pending:
            now = clock()
            if now > wall_limit:
                break
            r = pending[0]
            if r.arrival > now:
                time.sleep(min(r.arrival - now, 0.01))
                continue
            pending.popleft()
            r.start = clock()
            if r.kind == "render":
                img = self.render_targets[r.payload].render()
                r.result = img.cpu()
            else:
                prob = upload(self.pose_payloads[r.payload], self.dev)
                xi, _ = pose_mod.solve(prob, iters=self.iters, mode=self.mode)
                r.result = xi
            torch.cuda.synchronize(self.dev)
            r.done = clock()
            stats.completed.append(r)
            stats.admitted_peak = 1
        stats.wall = clock()
        return stats
