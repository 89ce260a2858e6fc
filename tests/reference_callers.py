"""Running the reference's own render callers on the CPU, unchanged, through this
package's drop-in `diff_gaussian_rasterization` — test infrastructure.

The callers are CF3DGS_Render.render (scene/gaussian_model_cf.py:777-910) and
gaussian_renderer.render (gaussian_renderer/__init__.py:19-113). Importing them needs
modules that are not installed here; they are stubbed in sys.modules (lietorch,
simple_knn._C, plyfile, PIL, matplotlib, mpl_toolkits: none of them is used on the
render path). The callers place tensors on "cuda"; this machine has no GPU, so tensor
factories are pointed at the CPU while the callers run. The drop-in package itself runs
unmodified — settings NamedTuple, argument validation, autograd Function — except for
its two native calls (cfgs.raster.forward / backward), which the CPU test replaces with
the C oracle; on a GPU the same package runs the CUDA kernels, and
tests/test_reference_callers_gpu.py replays the recorded calls there.

The reference tree is read from CFGS_REFERENCE_ROOT (default: the survey machine's
checkout); everything here skips when it is absent (it is not present on GPU machines).
"""
from __future__ import annotations

import contextlib
import math
import os
import sys
import types

import numpy as np
import torch

REFERENCE_ROOT = os.environ.get("CFGS_REFERENCE_ROOT", "/root/reference")


def available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "scene", "gaussian_model_cf.py"))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


class _Unused:
    """Stands in for an attribute of a stubbed module; fails loudly if the render path
    ever touches it."""

    def __init__(self, name):
        self.name = name

    def __call__(self, *a, **k):
        raise RuntimeError(f"{self.name} is stubbed and not part of the render path")

    def __getattr__(self, item):
        raise RuntimeError(f"{self.name}.{item} is stubbed and not part of the render path")


def _stubs() -> dict:
    u = _Unused
    mpl = _stub("matplotlib", use=lambda *a, **k: None, cm=u("matplotlib.cm"))
    plt = _stub("matplotlib.pyplot")
    mpl.pyplot = plt
    return {
        "lietorch": _stub("lietorch", SO3=u("SO3"), SE3=u("SE3"), Sim3=u("Sim3"),
                          LieGroupParameter=u("LieGroupParameter")),
        "simple_knn": _stub("simple_knn"),
        "simple_knn._C": _stub("simple_knn._C", distCUDA2=u("distCUDA2")),
        "plyfile": _stub("plyfile", PlyData=u("PlyData"), PlyElement=u("PlyElement")),
        "PIL": _stub("PIL", Image=u("PIL.Image")),
        "PIL.Image": _stub("PIL.Image"),
        "matplotlib": mpl,
        "matplotlib.pyplot": plt,
        "matplotlib.patches": _stub("matplotlib.patches", Patch=u("Patch")),
        "mpl_toolkits": _stub("mpl_toolkits"),
        "mpl_toolkits.mplot3d": _stub("mpl_toolkits.mplot3d"),
        "mpl_toolkits.mplot3d.art3d": _stub("mpl_toolkits.mplot3d.art3d", Poly3DCollection=u("Poly3DCollection")),
    }


def _cpu_device(kw):
    d = kw.get("device")
    if d is not None and str(d).startswith("cuda"):
        kw["device"] = "cpu"
    return kw


@contextlib.contextmanager
def reference_modules():
    """Imports the two callers (with the stubs and the CPU device redirect in place) and
    yields (scene.gaussian_model_cf module, gaussian_renderer module)."""
    saved_mods = {k: sys.modules.get(k) for k in list(_stubs())}
    saved_path = list(sys.path)
    names = ("zeros_like", "tensor", "zeros", "ones", "empty", "full", "eye")
    factories = {n: getattr(torch, n) for n in names}
    try:
        sys.modules.update(_stubs())
        sys.path.insert(0, REFERENCE_ROOT)
        for n, f in factories.items():
            setattr(torch, n, (lambda f_: lambda *a, **k: f_(*a, **_cpu_device(k)))(f))
        import importlib
        gm = importlib.import_module("scene.gaussian_model_cf")
        gr = importlib.import_module("gaussian_renderer")
        yield gm, gr
    finally:
        for n, f in factories.items():
            setattr(torch, n, f)
        sys.path[:] = saved_path
        for k, v in saved_mods.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
        for k in [k for k in sys.modules if k == "scene" or k.startswith("scene.") or k == "gaussian_renderer"
                  or k == "utils" or k.startswith("utils.")]:
            sys.modules.pop(k, None)


class Camera:
    """The attributes the callers read from a viewpoint camera (scene/cameras.py:57-74)."""

    def __init__(self, cam, uid=0):
        self.FoVx = 2.0 * math.atan(cam.tanfovx)
        self.FoVy = 2.0 * math.atan(cam.tanfovy)
        self.image_width, self.image_height = cam.width, cam.height
        self.world_view_transform = cam.viewmatrix
        self.full_proj_transform = cam.projmatrix
        self.camera_center = cam.campos
        self.uid = uid


class Pipe:
    def __init__(self, compute_cov3D_python=False, convert_SHs_python=False, debug=False):
        self.compute_cov3D_python = compute_cov3D_python
        self.convert_SHs_python = convert_SHs_python
        self.debug = debug


def load_scene_into(model, scene):
    """Sets a CFGaussianModel's raw parameters so that its activations (exp, sigmoid,
    normalize) give the scene's Gaussians."""
    from torch import nn
    p = lambda t: nn.Parameter(t.detach().clone().contiguous().requires_grad_(True))
    model._xyz = p(scene.means3D)
    model._features_dc = p(scene.shs[:, :1, :])
    model._features_rest = p(scene.shs[:, 1:, :])
    model._scaling = p(torch.log(scene.scales))
    model._rotation = p(scene.rotations)
    o = scene.opacities.double().clamp(1e-6, 1 - 1e-6)
    model._opacity = p(torch.log(o / (1 - o)).float())
    model.active_sh_degree = scene.sh_degree
    model.max_sh_degree = scene.sh_degree
    model.rotate_xyz = False
    model.rotate_seq = False


class OracleRaster:
    """Replacement of cfgs.raster.forward / backward by the C oracle (CPU), recording
    every call the drop-in makes: the settings and the tensors the reference passed."""

    def __init__(self):
        self.calls = []

    def forward(self, rs, means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp, timers=None):
        from oracle.c_oracle import Oracle
        o = Oracle(rs.image_width, rs.image_height, rs.tanfovx, rs.tanfovy, rs.bg, rs.scale_modifier, rs.viewmatrix,
                   rs.projmatrix, rs.sh_degree, rs.campos, means3D, opacities, shs=shs, colors_precomp=colors_precomp,
                   scales=scales, rotations=rotations, cov3D_precomp=cov3D_precomp).forward()
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
        rec = {"settings": {k: (v.detach().clone() if isinstance(v, torch.Tensor) else v)
                            for k, v in rs._asdict().items()},
               "inputs": {k: (None if v is None else v.detach().clone())
                          for k, v in dict(means3D=means3D, opacities=opacities, shs=shs,
                                           colors_precomp=colors_precomp, scales=scales, rotations=rotations,
                                           cov3D_precomp=cov3D_precomp).items()}}
        self.calls.append(rec)
        return t(o.color), t(o.radii), t(o.depth), t(o.alpha), o

    def backward(self, rs, state, means3D, opacities, shs, colors_precomp, scales, rotations, cov3D_precomp,
                 grad_color, grad_depth, grad_alpha, timers=None):
        g = state.backward(grad_color.detach().numpy(),
                           None if grad_depth is None else grad_depth.detach().numpy(),
                           None if grad_alpha is None else grad_alpha.detach().numpy())
        self.calls[-1]["grads_in"] = {"color": grad_color.detach().clone(),
                                      "depth": None if grad_depth is None else grad_depth.detach().clone(),
                                      "alpha": None if grad_alpha is None else grad_alpha.detach().clone()}
        t = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a))
        return (t(g["means2D"]), t(g["colors"]), t(g["opacity"]), t(g["means3D"]), t(g["cov3D"]), t(g["sh"]),
                t(g["scales"]), t(g["rotations"]))
