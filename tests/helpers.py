"""Shared helpers of the test suite."""
from __future__ import annotations

import numpy as np
import torch


def settings_for(dgr, scene, device="cuda", bg=None, scale_modifier=1.0, prefiltered=False, debug=False,
                 sh_degree=None):
    cam = scene.camera.to(device)
    return dgr.GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy,
        bg=(scene.bg if bg is None else bg).to(device), scale_modifier=scale_modifier,
        viewmatrix=cam.viewmatrix, projmatrix=cam.projmatrix,
        sh_degree=scene.sh_degree if sh_degree is None else sh_degree, campos=cam.campos,
        prefiltered=prefiltered, debug=debug)


def grad_close(got, want, rtol=1e-4, floor=1e-2):
    """Element-wise relative check with a floor: |got - want| <= rtol * (|want| +
    floor * max|want|). The floor keeps elements that are sums with cancellation (near
    zero relative to the tensor's scale) from demanding more than float32 summation in a
    different order can give. Returns (ok, worst ratio)."""
    got = np.asarray(got, np.float64).reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    if want.size == 0:
        return True, 0.0
    scale = float(np.abs(want).max())
    if scale == 0.0:
        return bool(np.abs(got).max() == 0.0), float(np.abs(got).max())
    bound = rtol * (np.abs(want) + floor * scale)
    ratio = np.abs(got - want) / bound
    return bool((ratio <= 1.0).all()), float(ratio.max())


def assert_grad_close(name, got, want, rtol=1e-4, floor=1e-2):
    ok, worst = grad_close(got, want, rtol, floor)
    assert ok, f"{name}: worst |err| / (rtol*(|ref| + floor*max|ref|)) = {worst:.3g} (> 1)"


def grad_report(got, want, bound, rtol=1e-4) -> dict:
    """How `got` (float32 kernels) compares with the float64 oracle `want`: the fraction
    of elements within rtol relative with no floor, the worst relative error, and the
    worst ratio of the error to rtol |want| + bound (bound: the per-element float32
    rounding bound of oracle.error_bound)."""
    got = np.asarray(got, np.float64).reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    b = np.asarray(bound, np.float64).reshape(-1)
    err = np.abs(got - want)
    if want.size == 0:
        return {"n": 0}
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(err == 0, 0.0, err / np.abs(want))
        ratio = np.where(err == 0, 0.0, err / (rtol * np.abs(want) + b))
        brel = np.where(b == 0, 0.0, b / np.abs(want))
    return {"n": int(want.size), "within_rtol": float((rel <= rtol).mean()), "max_rel": float(np.nanmax(rel)),
            "max_err_over_tol": float(np.nanmax(ratio)), "median_bound_rel": float(np.nanmedian(brel))}


def assert_grad_bounded(name, got, want, bound, rtol=1e-4):
    """Elementwise |got - want| <= rtol |want| + bound: within 1e-4 relative, or, where the
    float32 computation cannot reach that (its terms cancel), within the float32 rounding
    bound of the same computation (oracle.error_bound.backward_bounds) — no floor taken
    from the tensor's largest element."""
    got = np.asarray(got, np.float64).reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    b = np.asarray(bound, np.float64).reshape(-1)
    err = np.abs(got - want)
    tol = rtol * np.abs(want) + b
    bad = ~(err <= tol)
    if bad.any():
        i = int(np.argmax(np.where(bad, err / np.maximum(tol, 1e-300), 0)))
        raise AssertionError(f"{name}: {int(bad.sum())} of {want.size} elements outside rtol |ref| + float32 bound; "
                             f"worst at {i}: got {got[i]:.9g} want {want[i]:.9g} bound {b[i]:.3g}")


def bits(a):
    return np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32)


def l1_image_grad(color: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """dL/dcolor of L = mean |clamp(color, 0, 1) - target| (the CF-3DGS RGB L1,
    trainer/losses.py:98-136 with lambda_dssim = 0, after the clamp of
    scene/gaussian_model_cf.py:885), with torch's subgradient conventions."""
    c = color.detach()
    inside = ((c >= 0) & (c <= 1)).to(c.dtype)
    return torch.sign(c.clamp(0, 1) - target) * inside / c.numel()
