"""Generates tests/golden/reference_math.npz by running the reference's own Python
functions (CF-3DGS repository, mounted read-only at the path given on the command line
or in CFGS_REFERENCE) on seeded inputs:

- utils/sh_utils.py eval_sh (degrees 0..3) at random unit directions, and the colour
  the renderer derives from it, clamp_min(eval_sh + 0.5, 0)
  (scene/gaussian_model_cf.py:861-864);
- utils/general_utils.py build_rotation, build_scaling_rotation and strip_symmetric,
  i.e. the 3D covariance the rasteriser computes from scales and quaternions
  (scene/gaussian_model_cf.py:834-838);
- scene/cameras.py Camera (intrinsics branch) with utils/graphics_utils.py
  getWorld2View3: world_view_transform, full_proj_transform, camera_center;
- utils/graphics_utils.py getProjectionMatrix / fov2focal / focal2fov;
- utils/loss_utils.py ssim (the pose loss's SSIM term) on seeded image pairs, with
  autograd's gradient with respect to the first image.

The reference writes device='cuda' into some tensor constructors and calls .cuda();
this script runs them on the CPU by dropping those device arguments. Run:
    python tests/golden/make_golden.py /path/to/CF-3DGS
"""
import os
import sys
import types

import numpy as np
import torch

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CFGS_REFERENCE", "")
if not REF or not os.path.isdir(REF):
    raise SystemExit("usage: make_golden.py <reference checkout>")
sys.path.insert(0, REF)

from utils import sh_utils, general_utils, graphics_utils  # noqa: E402

# CPU shims for the reference's hard-coded CUDA placement
_zeros = torch.zeros
shim = types.ModuleType("torch_cpu_shim")
shim.__dict__.update({k: getattr(torch, k) for k in dir(torch) if not k.startswith("__")})
shim.zeros = lambda *a, **k: _zeros(*a, **{kk: vv for kk, vv in k.items() if kk != "device"})
general_utils.torch = shim
torch.Tensor.cuda = lambda self, *a, **k: self
import importlib.util  # noqa: E402

# scene/cameras.py alone (the scene package's __init__ pulls in dataset readers)
_spec = importlib.util.spec_from_file_location("ref_cameras", os.path.join(REF, "scene", "cameras.py"))
cameras = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(cameras)

rng = np.random.default_rng(1234)
out = {}

# SH
n = 64
dirs = rng.standard_normal((n, 3))
dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
sh = rng.normal(0, 0.5, (n, 16, 3))
out["sh_dirs"] = dirs.astype(np.float32)
out["sh_coeffs"] = sh.astype(np.float32)  # [N, 16, 3] as the rasteriser takes them
for deg in range(4):
    shs_view = torch.tensor(sh, dtype=torch.float64).transpose(1, 2)  # [N, 3, 16] as eval_sh takes them
    r = sh_utils.eval_sh(deg, shs_view, torch.tensor(dirs))
    out[f"sh_eval_deg{deg}"] = r.numpy()
    out[f"sh_color_deg{deg}"] = torch.clamp_min(r + 0.5, 0.0).numpy()

# covariance from scale and quaternion
s = np.exp(rng.normal(-3.0, 0.7, (n, 3)))
q = rng.standard_normal((n, 4))
q /= np.linalg.norm(q, axis=1, keepdims=True)
out["cov_scales"] = s.astype(np.float32)
out["cov_rotations"] = q.astype(np.float32)
for mod in (1.0, 0.7):
    L = general_utils.build_scaling_rotation(mod * torch.tensor(s, dtype=torch.float32),
                                             torch.tensor(q, dtype=torch.float32))
    cov = general_utils.strip_symmetric(L @ L.transpose(1, 2))
    out[f"cov3d_mod{mod}"] = cov.numpy()

# cameras (intrinsics branch of scene/cameras.py)
cams = []
for i in range(4):
    W, H = [(256, 256), (1920, 1080), (640, 360), (97, 61)][i]
    fx = fy = [256.0, 1400.0, 500.0, 80.0][i]
    cx, cy = W / 2.0 + (3.5 if i == 3 else 0.0), H / 2.0 - (2.0 if i == 3 else 0.0)
    ang = rng.uniform(0, 0.3)
    axis = rng.standard_normal(3)
    axis /= np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
    T = rng.normal(0, 0.5, 3)
    intr = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1]], dtype=np.float64)
    img = torch.zeros(3, H, W)
    c = cameras.Camera(0, R, T, graphics_utils.focal2fov(fx, W), graphics_utils.focal2fov(fy, H), img, None, "x", 0,
                       intrinsics=intr, data_device="cpu", is_co3d=True)
    out[f"cam{i}_R"] = R
    out[f"cam{i}_T"] = T
    out[f"cam{i}_intr"] = np.array([W, H, fx, fy, cx, cy])
    out[f"cam{i}_view"] = c.world_view_transform.numpy()
    out[f"cam{i}_full"] = c.full_proj_transform.numpy()
    out[f"cam{i}_center"] = c.camera_center.numpy()
    out[f"cam{i}_tanfov"] = np.array([np.tan(c.FoVx * 0.5), np.tan(c.FoVy * 0.5)])

# projection matrix from field of view
P = graphics_utils.getProjectionMatrix(0.01, 100.0, 1.1, 0.8)
out["projmatrix_fov"] = P.numpy()
out["fov2focal"] = np.array([graphics_utils.fov2focal(1.1, 640), graphics_utils.focal2fov(500.0, 640)])

# SSIM (utils/loss_utils.py:33-58), float64, gradient by autograd
from utils import loss_utils  # noqa: E402
for i, (C, H, W) in enumerate([(3, 24, 31), (1, 13, 9), (3, 40, 64)]):
    a = rng.uniform(0, 1, (C, H, W))
    b = np.clip(a + rng.normal(0, 0.15, (C, H, W)), 0, 1) if i != 1 else rng.uniform(0, 1, (C, H, W))
    x = torch.tensor(a[None], dtype=torch.float64, requires_grad=True)
    win = loss_utils.create_window(11, C).double()
    v = loss_utils._ssim(x, torch.tensor(b[None], dtype=torch.float64), win, 11, C, True)
    v.backward()
    out[f"ssim{i}_img1"] = a.astype(np.float32)
    out[f"ssim{i}_img2"] = b.astype(np.float32)
    out[f"ssim{i}_value"] = np.array(v.item())
    out[f"ssim{i}_grad"] = x.grad[0].numpy()

dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_math.npz")
np.savez_compressed(dst, **out)
print("wrote", dst, sum(v.nbytes for v in out.values()), "bytes")
