"""Batched CF-3DGS pose solves on one GPU.

Many relative-pose solves (trainer/cf3dgs_trainer.py:261-285 each: 300 Adam iterations
of the SE(3) tangent on the RGB L1 of the clamped render) advance together: one
cfgs_batch_iteration call runs one iteration of every solve with one kernel launch per
stage, and a run of iterations is captured once in a CUDA graph and replayed. Per
solve the arithmetic is that of the single fused solve (cfgs.pose.solve(mode="fused")),
so a solve's result is the same alone, in any batch, and in the single-solve path.
The render schedule (cfgs.autotune) can be tuned per batch shape; every schedule gives
the same bits.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import autotune as autotune_mod
from . import native
from .pose import PoseProblem

_SLOT = 256  # Gaussian slots are allocated per solve in multiples of the 256-wide block


@dataclass
class BatchResult:
    xi: np.ndarray            # [S,6] float64 copies of the final float32 tangents
    iterations: int
    seconds: float            # wall time of the timed iterations (graph replays)
    capacity: int
    num_rendered0: int        # K of the first iteration (all solves together)
    overflowed: bool
    retries: int


def _raise_on_timeout(flags: int) -> None:
    """A kernel's bounded wait (for an on-chip copy, or the one-launch binning's wait
    for the other blocks) ran out: the iterations' results are invalid."""
    if flags & (native.FLAG_COPY_TIMEOUT | native.FLAG_BARRIER_TIMEOUT):
        raise RuntimeError(f"a bounded device wait ran out (flags 0x{flags:x}); the batch's results are invalid")


class BatchSolver:
    """Packs `problems` (device-resident PoseProblem objects with equal SH width) into
    one batch. Call solve(iters) to run them."""

    def __init__(self, problems: list[PoseProblem], lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-15,
                 capacity_factor: float = 1.25, graph_chunk: int = 25, use_graph: bool = True, autotune=None):
        """autotune: None (keep the process-wide render schedule), True (tune with the
        default cache) or an autotune.Autotuner; when set, the render schedule of this
        batch's shape is looked up or tuned on the batch itself before its iterations."""
        if not problems:
            raise ValueError("empty batch")
        self.problems = problems
        self.tuner = (autotune_mod.Autotuner() if autotune is True else autotune) or None
        self.schedule = None
        self.dev = problems[0].xyz.device
        self.lr, self.betas, self.eps = float(lr), betas, float(eps)
        self.capacity_factor = capacity_factor
        self.graph_chunk = graph_chunk
        self.use_graph = use_graph
        self.lib = native.load()
        M = {int(p.shs.shape[1]) for p in problems}
        if len(M) != 1:
            raise ValueError("all solves in a batch must have the same number of SH coefficients")
        self.M = M.pop()
        self._plan()
        self._pack()

    # ---- layout --------------------------------------------------------------------
    def _plan(self):
        S = len(self.problems)
        self.S = S
        scenes = (native.BatchScene * S)()
        self._keep = []
        for s, p in enumerate(self.problems):
            rs = p.settings
            view = rs.viewmatrix.float().contiguous()
            proj = rs.projmatrix.float().contiguous()
            campos = rs.campos.float().contiguous()
            bg = rs.bg.float().contiguous()
            self._keep += [view, proj, campos, bg]
            sc = scenes[s]
            sc.image_width, sc.image_height = int(rs.image_width), int(rs.image_height)
            sc.tanfovx, sc.tanfovy = float(rs.tanfovx), float(rs.tanfovy)
            sc.viewmatrix, sc.projmatrix = view.data_ptr(), proj.data_ptr()
            sc.campos, sc.bg = campos.data_ptr(), bg.data_ptr()
            sc.sh_degree, sc.sh_coeffs = int(rs.sh_degree), self.M
            sc.num_gaussians = int(p.xyz.shape[0])
        self.scenes = scenes
        plan = native.BatchPlan()
        native.check(self.lib.cfgs_batch_plan(S, scenes, None, C.byref(plan), None, None, None, None, None, None),
                     "cfgs_batch_plan")
        self.pose_states = torch.zeros(plan.pose_state_bytes, dtype=torch.uint8, device=self.dev)
        desc = np.zeros(plan.desc_bytes, np.uint8)
        block_scene = np.zeros(plan.num_blocks, np.int32)
        tile_scene = np.zeros(plan.num_tiles, np.int32)
        gb = np.zeros(S, np.int32)
        tb = np.zeros(S, np.int32)
        pb = np.zeros(S, np.int64)
        ptr = lambda a: a.ctypes.data
        native.check(self.lib.cfgs_batch_plan(S, scenes, self.pose_states.data_ptr(), C.byref(plan), ptr(desc),
                                              ptr(block_scene), ptr(tile_scene), ptr(gb), ptr(tb), ptr(pb)),
                     "cfgs_batch_plan")
        self.plan = plan
        self.gauss_base, self.tile_base, self.pix_base = gb, tb, pb
        self.descs = torch.from_numpy(desc).to(self.dev)
        self.block_scene = torch.from_numpy(block_scene).to(self.dev)
        self.tile_scene = torch.from_numpy(tile_scene).to(self.dev)

    def _pack(self):
        dev, plan, M = self.dev, self.plan, self.M
        slots = plan.gauss_slots
        f = dict(device=dev, dtype=torch.float32)
        self.means = torch.zeros(slots, 3, **f)
        self.opac = torch.zeros(slots, **f)
        self.shs = torch.zeros(slots, M, 3, **f)
        self.scales = torch.ones(slots, 3, **f)
        self.rots = torch.zeros(slots, 4, **f)
        self.rots[:, 0] = 1.0
        self.target = torch.zeros(3 * plan.num_pixels, **f)
        self.color = torch.zeros(3 * plan.num_pixels, **f)
        for s, p in enumerate(self.problems):
            g0, n = int(self.gauss_base[s]), int(p.xyz.shape[0])
            self.means[g0:g0 + n] = p.xyz
            self.opac[g0:g0 + n] = p.opacities.reshape(-1)
            self.shs[g0:g0 + n] = p.shs
            self.scales[g0:g0 + n] = p.scales
            self.rots[g0:g0 + n] = p.rotations
            q0 = 3 * int(self.pix_base[s])
            self.target[q0:q0 + p.target.numel()] = p.target.reshape(-1)
        self.radii = torch.zeros(slots, dtype=torch.int32, device=dev)
        self.geom = torch.zeros(plan.geom_bytes, dtype=torch.uint8, device=dev)
        self.image = torch.zeros(plan.image_bytes, dtype=torch.uint8, device=dev)
        self.partials = torch.zeros(plan.num_blocks * 9, dtype=torch.float64, device=dev)
        self.xi = torch.zeros(self.S, 6, **f)
        self.adam = torch.zeros(self.S, 16, **f)
        self._alloc_instances(0)

    def _alloc_instances(self, capacity: int):
        self.capacity = int(capacity)
        self.binning = torch.empty(self.lib.cfgs_binning_bytes(self.capacity), dtype=torch.uint8, device=self.dev)
        self.scratch = torch.empty(self.lib.cfgs_backward_scratch_bytes(self.capacity), dtype=torch.uint8,
                                   device=self.dev)

    def _args(self) -> native.BatchArgs:
        a = native.BatchArgs()
        p = self.plan
        a.num_scenes, a.num_blocks, a.num_tiles = self.S, p.num_blocks, p.num_tiles
        a.gauss_slots, a.capacity = p.gauss_slots, self.capacity
        a.descs, a.block_scene, a.tile_scene = self.descs.data_ptr(), self.block_scene.data_ptr(), \
            self.tile_scene.data_ptr()
        a.means3D, a.opacities, a.shs = self.means.data_ptr(), self.opac.data_ptr(), self.shs.data_ptr()
        a.scales, a.rotations = self.scales.data_ptr(), self.rots.data_ptr()
        a.target, a.color, a.radii = self.target.data_ptr(), self.color.data_ptr(), self.radii.data_ptr()
        a.geom, a.image = self.geom.data_ptr(), self.image.data_ptr()
        a.binning, a.scratch = self.binning.data_ptr(), self.scratch.data_ptr()
        a.pose_partials, a.xi, a.adam_state = self.partials.data_ptr(), self.xi.data_ptr(), self.adam.data_ptr()
        a.pose_states = self.pose_states.data_ptr()
        a.lr, a.beta1, a.beta2, a.eps = self.lr, float(self.betas[0]), float(self.betas[1]), self.eps
        # this batch's tuned schedule, else the calling thread's current one
        a.schedule = autotune_mod.c_schedule(self.schedule)
        a.sh_degree_bound = 1 + max(int(sc.sh_degree) for sc in self.scenes)
        return a

    def _counts(self) -> native.Counts:
        c = native.Counts()
        native.check(self.lib.cfgs_read_counts(self.image.data_ptr(), C.byref(c),
                                               torch.cuda.current_stream(self.dev).cuda_stream), "cfgs_read_counts")
        return c

    def reset(self):
        self.xi.zero_()
        self.adam.zero_()

    def load_state(self, xi: torch.Tensor, adam: torch.Tensor):
        """Sets every solve's tangent [S,6] and Adam state [S,16] (to resume solves)."""
        self.xi.copy_(xi)
        self.adam.copy_(adam)

    def _apply_schedule(self) -> None:
        """Sets this batch's render schedule for its shape (tuning it on the batch when
        the cache has none); the solves' state is left as it was. Without a tuner the
        batch uses the calling thread's current schedule."""
        if self.tuner is None:
            return
        key = autotune_mod.batch_key(int(sum(int(p.xyz.shape[0]) for p in self.problems)), int(self.plan.num_tiles),
                                     self.M)
        sched = self.tuner.lookup(key)
        if sched is None:
            saved = (self.xi.clone(), self.adam.clone())
            dev = self.dev
            self.schedule = None
            args = self._args()

            def run():  # one iteration under the schedule the tuner is timing (this thread's)
                args.schedule = autotune_mod.c_schedule()
                native.check(self.lib.cfgs_batch_iteration(C.byref(args), torch.cuda.current_stream(dev).cuda_stream),
                             "cfgs_batch_iteration")

            native.check(self.lib.cfgs_batch_init(C.byref(args), torch.cuda.current_stream(dev).cuda_stream),
                         "cfgs_batch_init")
            sched = self.tuner.tune(key, run)
            self.load_state(*saved)
        self.schedule = sched

    def launch(self, iters: int) -> torch.cuda.Event:
        """Enqueues `iters` iterations of every solve from the current state (no reset)
        and returns an event that completes with them. The first call sizes the
        instance capacity from the current poses (one counting iteration)."""
        self._saved = (self.xi.clone(), self.adam.clone(), iters)
        if getattr(self, "_cap_ready", False) is False:
            K0 = self.probe_capacity()
            self.load_state(self._saved[0], self._saved[1])
            self._alloc_instances(int(K0 * self.capacity_factor) + 4096)
            self._cap_ready = True
        self._apply_schedule()
        args = self._args()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        native.check(self.lib.cfgs_batch_init(C.byref(args), st), "cfgs_batch_init")
        done = self._run_graph(args, iters) if (self.use_graph and iters >= self.graph_chunk) else 0
        for _ in range(iters - done):
            native.check(self.lib.cfgs_batch_iteration(C.byref(args), st), "cfgs_batch_iteration")
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.dev))
        return ev

    def finish(self) -> bool:
        """After launch()'s event: True if the iterations ran within capacity; otherwise
        restores the state saved by launch() and doubles the capacity (re-launch)."""
        flags = self._counts().flags
        _raise_on_timeout(flags)
        if not (flags & native.FLAG_CAPACITY_OVERFLOW):
            return True
        self.load_state(self._saved[0], self._saved[1])
        self._alloc_instances(self.capacity * 2)
        return False

    def run(self, iters: int) -> bool:
        """launch() + finish(), retrying with more capacity up to three times."""
        for _ in range(4):
            self.launch(iters).synchronize()
            if self.finish():
                return True
        return False

    # ---- running -------------------------------------------------------------------
    def prepare(self) -> native.BatchArgs:
        """Resets every solve, sizes the instance capacity from a counting iteration and
        initialises the pose states; returns the arguments for iterate()."""
        K0 = self.probe_capacity()
        self.reset()
        self._alloc_instances(int(K0 * self.capacity_factor) + 4096)
        args = self._args()
        native.check(self.lib.cfgs_batch_init(C.byref(args), torch.cuda.current_stream(self.dev).cuda_stream),
                     "cfgs_batch_init")
        return args

    def iterate(self, args: native.BatchArgs) -> None:
        """Enqueues one iteration of every solve (eager launches, no graph)."""
        native.check(self.lib.cfgs_batch_iteration(C.byref(args), torch.cuda.current_stream(self.dev).cuda_stream),
                     "cfgs_batch_iteration")

    def probe_capacity(self) -> int:
        """K of the current poses (an iteration at capacity 0 only counts; the update
        is skipped), and a capacity with headroom for the poses to move."""
        if self.capacity != 0:
            self._alloc_instances(0)
        args = self._args()
        st = torch.cuda.current_stream(self.dev).cuda_stream
        native.check(self.lib.cfgs_batch_init(C.byref(args), st), "cfgs_batch_init")
        native.check(self.lib.cfgs_batch_iteration(C.byref(args), st), "cfgs_batch_iteration")
        K = int(self._counts().num_rendered)
        return K

    def solve(self, iters: int = 300) -> BatchResult:
        retries = 0
        K0 = self.probe_capacity()
        cap = int(K0 * self.capacity_factor) + 4096
        while True:
            self.reset()
            self._alloc_instances(cap)
            self._apply_schedule()
            args = self._args()
            st = torch.cuda.current_stream(self.dev).cuda_stream
            native.check(self.lib.cfgs_batch_init(C.byref(args), st), "cfgs_batch_init")
            t0 = time.perf_counter()
            if self.use_graph and iters >= self.graph_chunk:
                done = self._run_graph(args, iters)
            else:
                done = 0
            for _ in range(iters - done):
                native.check(self.lib.cfgs_batch_iteration(C.byref(args), torch.cuda.current_stream(self.dev)
                                                           .cuda_stream), "cfgs_batch_iteration")
            torch.cuda.synchronize(self.dev)
            dt = time.perf_counter() - t0
            c = self._counts()
            _raise_on_timeout(c.flags)
            if c.flags & native.FLAG_CAPACITY_OVERFLOW and retries < 3:
                retries += 1
                cap *= 2
                continue
            return BatchResult(self.xi.double().cpu().numpy(), iters, dt, cap, K0,
                               bool(c.flags & native.FLAG_CAPACITY_OVERFLOW), retries)

    def _run_graph(self, args, iters: int) -> int:
        """Captures graph_chunk iterations into one CUDA graph and replays it; returns
        the number of iterations run."""
        chunk = self.graph_chunk
        # the first iteration runs outside the capture: the graph's memory must not be
        # the first use of any buffer (warm-up)
        s = torch.cuda.Stream(self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(chunk):
                    native.check(self.lib.cfgs_batch_iteration(C.byref(args), s.cuda_stream), "cfgs_batch_iteration")
        torch.cuda.current_stream(self.dev).wait_stream(s)
        n = iters // chunk
        for _ in range(n):
            g.replay()
        self._graph = g
        return n * chunk


def solve_sequential(problems: list[PoseProblem], iters: int = 300, mode: str = "plain"):
    """The comparison baseline: the solves one after another on the single-solve path."""
    from . import pose
    out, lat = [], []
    for p in problems:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xi, _ = pose.solve(p, iters=iters, mode=mode)
        torch.cuda.synchronize()
        lat.append(time.perf_counter() - t0)
        out.append(xi)
    return np.stack(out), lat
