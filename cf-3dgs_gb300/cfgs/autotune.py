"""Render-schedule autotuner.

The two per-tile render kernels have several launch shapes (CfgsRenderSchedule, a
field of every call's settings):
the forward's staging batch and warps per tile (4 warps on 8x8 pixel boxes with two
pixels per lane, or 8 warps on 8x4 boxes with one), and the backward's staging batch.
Every shape gives bit-identical results, so the choice only changes speed: the 4-warp
forward issues fewest instructions and wins when many tiles keep the GPU busy (a
1080p frame); with a few hundred tiles (one 640x360 pose solve) the GPU is
latency-bound and more, smaller warps can win.

The tuner times the candidates on the caller's own workload with CUDA events and keeps
the winner in a JSON cache keyed by the workload's shape — the Gaussian count rounded
up to a power of two, the image size (or, for a batch of solves, the tile count rounded
up to a power of two) and the SH width — so a shape is tuned once per cache.

The library keeps no schedule: each call carries one. On the host side the schedule
calls use is the calling thread's current one (set_schedule / using), so threads that
render different workloads with different schedules do not affect each other.
"""
from __future__ import annotations

import json
import os
import tempfile
import threading
from contextlib import contextmanager
from dataclasses import asdict, dataclass
from pathlib import Path
from typing import Callable

from . import native


@dataclass(frozen=True)
class Schedule:
    fwd_batch: int = 128
    fwd_warps: int = 4
    bwd_batch: int = 64
    bin_launch: int = 0  # batched solves: 0 one launch per binning stage, 1 one persistent launch


DEFAULT = Schedule()
FWD_CANDIDATES = [(128, 4), (64, 4), (256, 4), (128, 8), (256, 8)]  # (fwd_batch, fwd_warps), default first
BWD_CANDIDATES = [64, 32, 128]


_thread = threading.local()


def c_schedule(s: Schedule | None = None) -> "native.RenderSchedule":
    """The C struct of schedule s (default: the calling thread's current schedule)."""
    s = get_schedule() if s is None else s
    return native.RenderSchedule(s.fwd_batch, s.fwd_warps, s.bwd_batch, s.bin_launch)


def set_schedule(s: Schedule) -> None:
    """Makes s the schedule of the calling thread's later rasteriser calls (checked by the
    library: an unsupported shape raises)."""
    lib = native.load()
    native.check(lib.cfgs_render_schedule_check(native.C.byref(c_schedule(s)), None), "cfgs_render_schedule_check")
    _thread.schedule = s


def get_schedule() -> Schedule:
    """The calling thread's current schedule (DEFAULT until set)."""
    return getattr(_thread, "schedule", DEFAULT)


@contextmanager
def using(s: Schedule):
    """Runs the body under schedule s (in this thread) and restores the previous one."""
    old = get_schedule()
    set_schedule(s)
    try:
        yield s
    finally:
        set_schedule(old)


def bucket(n: int) -> int:
    """n rounded up to a power of two (1 for n <= 1)."""
    b = 1
    while b < n:
        b <<= 1
    return b


def raster_key(num_gaussians: int, width: int, height: int, sh_coeffs: int) -> str:
    return f"raster/n{bucket(num_gaussians)}/{width}x{height}/m{sh_coeffs}"


def batch_key(num_gaussians: int, num_tiles: int, sh_coeffs: int) -> str:
    return f"batch/n{bucket(num_gaussians)}/t{bucket(num_tiles)}/m{sh_coeffs}"


def default_cache_path() -> Path:
    env = os.environ.get("CFGS_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "cfgs" / "autotune.json"


def time_cuda(run: Callable[[], None], warmup: int = 2, iters: int = 10) -> float:
    """Milliseconds per call of run() on the current CUDA stream (events around `iters`
    calls after `warmup` untimed ones)."""
    import torch
    for _ in range(warmup):
        run()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record()
    for _ in range(iters):
        run()
    t1.record()
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / iters


class Autotuner:
    """Picks and caches render schedules. `measure(run, schedule) -> ms` times one
    candidate (CUDA events under that schedule by default; tests pass a fake)."""

    def __init__(self, path: str | Path | None = None,
                 measure: Callable[[Callable[[], None], Schedule], float] | None = None):
        self.path = Path(path) if path is not None else default_cache_path()
        self.measure = measure or self._measure_cuda
        self._cache = self._load()

    # ---- cache ---------------------------------------------------------------------
    def _load(self) -> dict:
        try:
            with open(self.path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    @staticmethod
    def _device() -> str:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.get_device_name(torch.cuda.current_device())
        except Exception:
            pass
        return "no-device"

    def full_key(self, key: str) -> str:
        """Cache entries are per GPU model: '<device name>|<workload key>'."""
        return f"{self._device()}|{key}"

    def lookup(self, key: str) -> Schedule | None:
        e = self._cache.get(self.full_key(key))
        if not isinstance(e, dict) or "schedule" not in e:
            return None
        try:
            return Schedule(**e["schedule"])
        except TypeError:
            return None

    def record(self, key: str, sched: Schedule, timings: dict) -> None:
        self._cache[self.full_key(key)] = {"schedule": asdict(sched), "ms": timings}
        self.path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=str(self.path.parent), prefix=".autotune.")
        with os.fdopen(fd, "w") as f:
            json.dump(self._cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    # ---- tuning --------------------------------------------------------------------
    @staticmethod
    def _measure_cuda(run: Callable[[], None], sched: Schedule) -> float:
        with using(sched):
            return time_cuda(run)

    def tune(self, key: str, run: Callable[[], None], force: bool = False, margin: float = 0.02) -> Schedule:
        """The cached schedule for `key`, or the best candidate on run() (one unit of the
        workload, enqueued on the current stream), recorded in the cache. Coordinate
        search: the forward shapes with the default backward batch, then the backward
        batches with the best forward shape. A candidate displaces the incumbent (the
        default first) only when it is faster by more than `margin`, and a choice other
        than the default must win again in an interleaved confirmation, so timing noise
        does not move the choice."""
        if not force:
            hit = self.lookup(key)
            if hit is not None:
                return hit
        timings: dict[str, float] = {}

        def trial(s: Schedule) -> float:
            ms = float(self.measure(run, s))
            timings[f"{s.fwd_batch}/{s.fwd_warps}/{s.bwd_batch}"] = round(ms, 5)
            return ms

        fwd_t = {fw: trial(Schedule(fw[0], fw[1], DEFAULT.bwd_batch)) for fw in FWD_CANDIDATES}
        best_fw = pick(FWD_CANDIDATES, fwd_t, margin)
        bwd_t = {b: fwd_t[best_fw] if b == DEFAULT.bwd_batch else trial(Schedule(best_fw[0], best_fw[1], b))
                 for b in BWD_CANDIDATES}
        chosen = Schedule(best_fw[0], best_fw[1], pick(BWD_CANDIDATES, bwd_t, margin))
        if chosen != DEFAULT:
            # confirmation: both timed twice more, interleaved; the challenger must still win
            # by the margin on the sum
            a = b = 0.0
            for _ in range(2):
                a += float(self.measure(run, DEFAULT))
                b += float(self.measure(run, chosen))
            timings["confirm_default"] = round(a / 2, 5)
            timings["confirm_chosen"] = round(b / 2, 5)
            if not b < a * (1.0 - margin):
                chosen = DEFAULT
        self.record(key, chosen, timings)
        return chosen


def pick(candidates: list, times: dict, margin: float):
    """The first candidate unless a later one is faster than the current best by more
    than the relative `margin`."""
    best = candidates[0]
    for c in candidates[1:]:
        if times[c] < times[best] * (1.0 - margin):
            best = c
    return best


def tune_rasterizer(raster_settings, means3D, opacities, shs=None, colors_precomp=None, scales=None,
                    rotations=None, cov3D_precomp=None, tuner: Autotuner | None = None,
                    apply: bool = True) -> Schedule:
    """Tunes the render schedule for one drop-in rasteriser workload (forward + backward
    with a unit image gradient) and, with apply=True, makes it the calling thread's
    schedule."""
    import torch
    from . import raster
    tuner = tuner or Autotuner()
    key = raster_key(int(means3D.shape[0]), int(raster_settings.image_width), int(raster_settings.image_height),
                     int(shs.shape[1]) if shs is not None else 0)
    grad = torch.full((3, int(raster_settings.image_height), int(raster_settings.image_width)),
                      1.0 / (3 * int(raster_settings.image_height) * int(raster_settings.image_width)),
                      device=means3D.device)

    def run():
        color, radii, depth, alpha, st = raster.forward(raster_settings, means3D, opacities, shs, colors_precomp,
                                                        scales, rotations, cov3D_precomp)
        raster.backward(raster_settings, st, means3D, opacities, shs, colors_precomp, scales, rotations,
                        cov3D_precomp, grad, None, None)

    sched = tuner.tune(key, run)
    if apply:
        set_schedule(sched)
    return sched
