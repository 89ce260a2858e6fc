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
import threading
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
    status: str = "pending"  # "ok", or why the request has no result: "rejected", "cancelled", "failed"
    error: str = ""

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
    per Gaussian for these scenes, 28 + 49 bytes each), and its render."""
    n = payload.xyz.shape[0]
    px = payload.target.numel() // 3
    return payload.nbytes + n * 64 + n * 2 * 77 + px * 3 * 4 * 2 + px * 8


def validate_payload(payload, hbm_budget: float = math.inf) -> str:
    """Why a pose request cannot be served ("" when it can): shapes and dtypes of the
    Gaussians and the target against the camera, a supported SH degree, finite values
    (CF-3DGS stops on a NaN loss, trainer/losses.py:126-127: a request that carries one
    is refused up front), and a device footprint within the HBM budget (a request that
    could never be admitted is refused instead of waiting forever)."""
    try:
        n = int(payload.xyz.shape[0])
        deg = int(payload.sh_degree)
        cam = payload.camera
        shapes = {"xyz": (payload.xyz, (n, 3)), "scales": (payload.scales, (n, 3)),
                  "rotations": (payload.rotations, (n, 4)), "target": (payload.target, (3, cam.height, cam.width))}
        if payload.xyz.dim() != 2 or n <= 0:
            return "xyz must be [N,3] with N > 0"
        if not 0 <= deg <= 3:
            return f"SH degree {deg} is not in 0..3"
        for name, (t, want) in shapes.items():
            if tuple(t.shape) != want:
                return f"{name} has shape {tuple(t.shape)}, expected {want}"
        if tuple(payload.opacities.reshape(-1).shape) != (n,):
            return f"opacities has {payload.opacities.numel()} values for {n} Gaussians"
        if payload.shs.dim() != 3 or payload.shs.shape[0] != n or payload.shs.shape[2] != 3 or \
                payload.shs.shape[1] < (deg + 1) ** 2:
            return f"shs has shape {tuple(payload.shs.shape)}, expected [{n}, >= {(deg + 1) ** 2}, 3]"
        for name in ("xyz", "opacities", "shs", "scales", "rotations", "target"):
            t = getattr(payload, name)
            if t.dtype != torch.float32:
                return f"{name} is {t.dtype}, expected float32"
            if not bool(torch.isfinite(t).all()):
                return f"{name} holds non-finite values"
    except (AttributeError, TypeError) as e:
        return f"malformed request: {e}"
    if solve_bytes(payload) > hbm_budget:
        return f"needs {solve_bytes(payload) / 1e9:.3f} GB, above the HBM budget of {hbm_budget / 1e9:.3f} GB"
    return ""


def _is_oom(e: BaseException) -> bool:
    return isinstance(e, torch.cuda.OutOfMemoryError) or (isinstance(e, RuntimeError) and "out of memory" in str(e))


@dataclass
class ServeStats:
    completed: list = field(default_factory=list)
    refused: list = field(default_factory=list)  # rejected, cancelled and failed requests
    wall: float = 0.0
    admitted_peak: int = 0
    epochs: int = 0

    def summary(self, name: str) -> dict:
        lat = np.array([r.latency for r in self.completed]) if self.completed else np.array([math.nan])
        kinds = {k: [r for r in self.completed if r.kind == k] for k in ("pose", "render")}
        pl = np.array([r.latency for r in kinds["pose"]]) if kinds["pose"] else np.array([math.nan])
        return {"server": name, "completed": len(self.completed), "wall_s": round(self.wall, 3),
                "rejected": sum(r.status == "rejected" for r in self.refused),
                "cancelled": sum(r.status == "cancelled" for r in self.refused),
                "failed": sum(r.status == "failed" for r in self.refused),
                "throughput_req_s": round(len(self.completed) / self.wall, 4) if self.wall else None,
                "pose_solves_per_s": round(len(kinds["pose"]) / self.wall, 4) if self.wall else None,
                "renders_per_s": round(len(kinds["render"]) / self.wall, 4) if self.wall else None,
                "latency_p50_s": round(float(np.nanpercentile(lat, 50)), 4),
                "latency_p99_s": round(float(np.nanpercentile(lat, 99)), 4),
                "pose_latency_p50_s": round(float(np.nanpercentile(pl, 50)), 4),
                "pose_latency_p99_s": round(float(np.nanpercentile(pl, 99)), 4),
                "peak_active_solves": self.admitted_peak, "epochs": self.epochs}


class ContinuousBatchServer:
    """Continuous batching of pose solves with renders on a side stream.

    Failure handling, each confined to the request concerned (the other solves keep their
    state and their results): a malformed request or one that could never fit the HBM
    budget is rejected on arrival (validate_payload); cancel(rid) withdraws a queued
    request, or an active solve at the next epoch boundary; a device allocation that
    fails while a solve is admitted fails that request (the server carries on); a solve
    whose pose turns non-finite is stopped at the next epoch boundary and failed (the
    reference stops on a NaN loss, trainer/losses.py:126-127). `hooks` lets a caller
    (tests) inject host-side faults: hooks["upload"](req) runs before a solve's inputs
    are copied to the device (it may raise), hooks["epoch"](batch_solver, requests)
    after every completed epoch."""

    def __init__(self, pose_payloads: list[PosePayload], render_targets: list[RenderTarget], device="cuda",
                 max_slots: int = 64, hbm_budget: float = 150e9, epoch: int = 25, iters: int = 300,
                 use_graph: bool = True, hooks: dict | None = None):
        self.pose_payloads = pose_payloads
        self.render_targets = render_targets
        self.dev = torch.device(device)
        self.max_slots, self.hbm_budget, self.epoch, self.iters = max_slots, hbm_budget, epoch, iters
        self.use_graph = use_graph
        self.hooks = dict(hooks or {})
        self._cancel_lock = threading.Lock()
        self._cancelled: set[int] = set()
        if iters % epoch:
            raise ValueError("iters must be a multiple of epoch")

    def cancel(self, rid: int) -> None:
        """Withdraws request `rid` (callable from any thread): dropped from the queue, or
        stopped at the next epoch boundary if it is running."""
        with self._cancel_lock:
            self._cancelled.add(int(rid))

    def _is_cancelled(self, rid: int) -> bool:
        with self._cancel_lock:
            return rid in self._cancelled

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

        def refuse(req, status, why):
            req.status, req.error, req.done = status, why, clock()
            stats.refused.append(req)

        def poll_renders():
            keep = []
            for req, ev, host in renders:
                if ev.query():
                    req.done = clock()
                    req.result = float(host.double().sum())  # the image reached the host
                    req.status = "ok"
                    pool.append(host)
                    stats.completed.append(req)
                else:
                    keep.append((req, ev, host))
            renders[:] = keep

        def ingest():
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                if r.kind == "pose":
                    if not 0 <= r.payload < len(self.pose_payloads):
                        refuse(r, "rejected", f"no pose payload {r.payload}")
                        continue
                    why = validate_payload(self.pose_payloads[r.payload], self.hbm_budget)
                    if why:
                        refuse(r, "rejected", why)
                    else:
                        queue.append(r)
                    continue
                if r.kind != "render" or not 0 <= r.payload < len(self.render_targets):
                    refuse(r, "rejected", f"unknown request {r.kind} / {r.payload}")
                    continue
                r.start = clock()
                with torch.cuda.stream(rstream):
                    img = self.render_targets[r.payload].render()
                    host = pool.pop() if pool else torch.empty(img.shape, dtype=img.dtype, pin_memory=True)
                    host.copy_(img, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(rstream)
                renders.append((r, ev, host))

        def drop(indices):
            """Removes active solves `indices` (their requests are settled), keeping the
            survivors' optimiser state."""
            nonlocal used
            if not indices:
                return
            if bs is not None and members == [id(x["req"]) for x in active]:
                for s, a in enumerate(active):
                    a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
            for s in sorted(indices, reverse=True):
                used -= active[s]["bytes"]
                del active[s]

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
                if "epoch" in self.hooks:
                    self.hooks["epoch"](bs, [a["req"] for a in active])
                finite = torch.isfinite(bs.xi).all(dim=1).cpu().tolist()
                gone = []
                for s, a in enumerate(active):
                    a["it"] += self.epoch
                    if not finite[s]:
                        refuse(a["req"], "failed", "the pose became non-finite (the loss diverged)")
                        gone.append(s)
                    elif self._is_cancelled(a["req"].rid):
                        refuse(a["req"], "cancelled", f"cancelled after {a['it']} iterations")
                        gone.append(s)
                    elif a["it"] >= self.iters:
                        a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
                        a["req"].result = a["xi"].double().cpu().numpy()
                        a["req"].done = clock()
                        a["req"].status = "ok"
                        stats.completed.append(a["req"])
                        gone.append(s)
                drop(gone)
            # epoch boundary: admission in arrival order, within slots and the HBM budget
            admitted = False
            while queue and len(active) < self.max_slots and clock() <= stop_admitting_after:
                r = queue[0]
                if self._is_cancelled(r.rid):
                    queue.popleft()
                    refuse(r, "cancelled", "cancelled while queued")
                    continue
                pl = self.pose_payloads[r.payload]
                need = solve_bytes(pl)
                if used + need > self.hbm_budget and active:
                    break
                queue.popleft()
                r.start = clock()
                if bs is not None and members == [id(a["req"]) for a in active]:
                    for s, a in enumerate(active):     # leaving the old batch: save its state
                        a["xi"], a["adam"] = bs.xi[s].clone(), bs.adam[s].clone()
                    members = None
                try:
                    if "upload" in self.hooks:
                        self.hooks["upload"](r)
                    prob = upload(pl, self.dev)
                except Exception as e:
                    if not _is_oom(e):
                        raise
                    refuse(r, "failed", f"device allocation failed: {e}")
                    torch.cuda.empty_cache()
                    continue
                active.append({"req": r, "prob": prob, "xi": torch.zeros(6, device=self.dev),
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
            why = ""
            if r.kind == "pose":
                why = validate_payload(self.pose_payloads[r.payload]) if 0 <= r.payload < len(self.pose_payloads) \
                    else f"no pose payload {r.payload}"
            elif r.kind != "render" or not 0 <= r.payload < len(self.render_targets):
                why = f"unknown request {r.kind} / {r.payload}"
            if why:
                r.status, r.error, r.done = "rejected", why, clock()
                stats.refused.append(r)
                continue
            if r.kind == "render":
                img = self.render_targets[r.payload].render()
                r.result = img.cpu()
            else:
                prob = upload(self.pose_payloads[r.payload], self.dev)
                xi, _ = pose_mod.solve(prob, iters=self.iters, mode=self.mode)
                r.result = xi
            torch.cuda.synchronize(self.dev)
            r.done = clock()
            r.status = "ok"
            stats.completed.append(r)
            stats.admitted_peak = 1
        stats.wall = clock()
        return stats
