"""Device-resident optimisation state of a Gaussian model (GaussianModel.training_setup,
the Adam step, add_densification_stats and densify_and_prune of
scene/gaussian_model_cf.py:242-301, 560-719) on libcfgs.so."""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import native
from .raster import _ptr, stream_handle

GROUPS = ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")


def _vp_array(ptrs):
    return (C.c_void_p * len(ptrs))(*ptrs)


class GaussianOptimizer:
    """params: {"xyz" [N,3], "f_dc" [N,1,3], "f_rest" [N,D-1,3], "opacity" [N,1],
    "scaling" [N,3], "rotation" [N,4]} float32 CUDA tensors (raw, pre-activation, as the
    reference stores them); lrs: per-group learning rates (training_setup)."""

    def __init__(self, params: dict, lrs: dict, betas=(0.9, 0.999), eps: float = 1e-15):
        self.params = {k: params[k].detach().float().contiguous() for k in GROUPS}
        self.lrs = {k: float(lrs[k]) for k in GROUPS}
        self.betas, self.eps = betas, float(eps)
        self.exp_avg = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.exp_avg_sq = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.step_count = 0
        n = self.num_gaussians
        dev = self.params["xyz"].device
        self.grad_accum = torch.zeros(n, dtype=torch.float32, device=dev)
        self.denom = torch.zeros(n, dtype=torch.float32, device=dev)
        self.max_radii2D = torch.zeros(n, dtype=torch.float32, device=dev)

    @property
    def num_gaussians(self) -> int:
        return int(self.params["xyz"].shape[0])

    def step(self, grads: dict) -> None:
        """One Adam step of every group (torch.optim.Adam(..., eps=1e-15) semantics)."""
        self.step_count += 1
        g = {k: grads[k].float().contiguous() for k in GROUPS}
        lib = native.load()
        args = [_vp_array([self.params[k].data_ptr() for k in GROUPS]), _vp_array([g[k].data_ptr() for k in GROUPS]),
                _vp_array([self.exp_avg[k].data_ptr() for k in GROUPS]),
                _vp_array([self.exp_avg_sq[k].data_ptr() for k in GROUPS]),
                (C.c_int64 * 6)(*[self.params[k].numel() for k in GROUPS]),
                (C.c_double * 6)(*[self.lrs[k] for k in GROUPS])]
        native.check(lib.cfgs_gaussian_adam(6, *args, self.betas[0], self.betas[1], self.eps, self.step_count,
                                            stream_handle(self.params["xyz"].device)), "cfgs_gaussian_adam")

    def add_densification_stats(self, grad_means2D: torch.Tensor, radii: torch.Tensor) -> None:
        g = grad_means2D.float().contiguous()
        r = radii.to(torch.int32).contiguous()
        native.check(native.load().cfgs_densify_stats(self.num_gaussians, _ptr(r), _ptr(g), _ptr(self.grad_accum),
                                                      _ptr(self.denom), stream_handle(g.device)), "cfgs_densify_stats")
        with torch.no_grad():
            self.max_radii2D = torch.where(r > 0, torch.maximum(self.max_radii2D, r.float()), self.max_radii2D)

    def densify_and_prune(self, max_grad: float, min_opacity: float, extent: float, max_screen_size,
                          percent_dense: float = 0.01, z: torch.Tensor | None = None,
                          generator: torch.Generator | None = None) -> dict:
        """densify_and_clone + densify_and_split + prune (scene/gaussian_model_cf.py:628-694).
        z: standard-normal draws [2, splits, 3] for the split children (drawn here when
        None). Returns the counts."""
        n = self.num_gaussians
        dev = self.params["xyz"].device
        lib = native.load()
        st = stream_handle(dev)
        ws = torch.empty(int(lib.cfgs_densify_workspace_bytes(n)), dtype=torch.uint8, device=dev)
        counts = (C.c_int64 * 4)()
        native.check(lib.cfgs_densify_plan(n, _ptr(self.grad_accum), _ptr(self.denom), _ptr(self.params["scaling"]),
                                           _ptr(self.params["opacity"]), float(max_grad), float(min_opacity),
                                           float(extent), float(percent_dense), 1 if max_screen_size else 0,
                                           _ptr(ws), counts, st), "cfgs_densify_plan")
        keep, clone, split, child = (int(c) for c in counts)
        if z is None:
            z = torch.randn((2, split, 3), device=dev, generator=generator)
        z = z.float().contiguous()
        rows = keep + clone + 2 * child
        xyz, scaling, rotation = self.params["xyz"], self.params["scaling"], self.params["rotation"]

        def write(src: torch.Tensor, role: int) -> torch.Tensor:
            w = src[0].numel() if src.shape[0] else int(math.prod(src.shape[1:]))
            out = torch.empty((rows,) + tuple(src.shape[1:]), dtype=torch.float32, device=dev)
            if n > 0 and rows > 0:
                native.check(lib.cfgs_densify_write(n, _ptr(ws), counts, int(w), _ptr(src), out.data_ptr(),
                                                    role, _ptr(xyz), _ptr(scaling), _ptr(rotation), _ptr(z), st),
                             "cfgs_densify_write")
            return out

        new_params = {k: write(v, {"xyz": 2, "scaling": 3}.get(k, 0)) for k, v in self.params.items()}
        self.exp_avg = {k: write(v, 1) for k, v in self.exp_avg.items()}
        self.exp_avg_sq = {k: write(v, 1) for k, v in self.exp_avg_sq.items()}
        self.params = new_params
        self.grad_accum = torch.zeros(rows, dtype=torch.float32, device=dev)
        self.denom = torch.zeros(rows, dtype=torch.float32, device=dev)
        self.max_radii2D = torch.zeros(rows, dtype=torch.float32, device=dev)
        return {"kept": keep, "cloned": clone, "split": split, "children_per_copy": child, "total": rows}
