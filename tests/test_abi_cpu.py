"""The C ABI library loads and exports every function include/cfgs.h and
include/cfgs_plain.h declare; host-side validation and workspace sizing work without a
GPU."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header: str):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cfgs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from cfgs import native
    lib = native.load()
    names = _declared("cfgs.h")
    assert len(names) >= 15
    plain = _declared("cfgs_plain.h")
    assert plain == ["cfgs_plain_backward", "cfgs_plain_bin", "cfgs_plain_render_forward", "cfgs_plain_work_bytes"]
    for n in names + plain:
        assert hasattr(lib, n), n
    assert set(native.EXPORTS) <= set(names) | set(plain)


def test_plain_path_rejects_invalid_arguments_on_host():
    from cfgs import native
    lib = native.load()
    assert lib.cfgs_plain_work_bytes(-1, 10, 64, 64) == 0
    assert lib.cfgs_plain_work_bytes(10, -1, 64, 64) == 0
    assert lib.cfgs_plain_work_bytes(10, 10, 0, 64) == 0
    assert lib.cfgs_plain_work_bytes(10, 1 << 31, 64, 64) == 0
    k = C.c_int64(-5)
    assert lib.cfgs_plain_bin(None, 10, 1, 1, 10, C.byref(k), None) == 1
    s = native.Settings()
    s.image_width, s.image_height = 64, 64
    assert lib.cfgs_plain_bin(C.byref(s), 10, 1, 1, 10, None, None) == 1
    assert lib.cfgs_plain_bin(C.byref(s), 10, 1, 1, 1 << 31, C.byref(k), None) == 5
    assert lib.cfgs_plain_bin(C.byref(s), 0, 1, 1, 10, C.byref(k), None) == 0 and k.value == 0
    assert lib.cfgs_plain_render_forward(C.byref(s), 10, 1, 1, 1, 10, None, None, None, None) == 1
    g = native.Gaussians()
    gr = native.Gradients()
    assert lib.cfgs_plain_backward(C.byref(s), C.byref(g), None, 1, 1, 1, 10, None, None, None, C.byref(gr),
                                   None) == 1


def test_workspace_sizes_and_layouts():
    from cfgs import native
    lib = native.load()
    assert lib.cfgs_geom_bytes(0) > 0
    g = native.geom_layout(1000)
    assert g["total"] == lib.cfgs_geom_bytes(1000)
    vals = [g[k] for k in native.GEOM_FIELDS]
    assert vals == sorted(vals) and all(v % 256 == 0 for v in vals)
    im = native.image_layout(1920, 1080)
    assert im["counts"] == 0  # raster.forward reads the counts from the workspace's first bytes
    assert im["total"] == lib.cfgs_image_bytes(1920, 1080)
    assert im["n_contrib"] - im["final_T"] >= 1920 * 1080 * 4
    b = native.binning_layout(12345)
    assert b["total"] == lib.cfgs_binning_bytes(12345)
    assert b["gid"] - b["key"] >= 12345 * 8 and b["sorted_pidx"] - b["sorted_gid"] >= 12345 * 4
    assert lib.cfgs_backward_scratch_bytes(1000) >= 1000 * 48
    assert lib.cfgs_image_bytes(0, 10) == 0


def test_invalid_arguments_rejected_on_host():
    """Argument checks run before any device work, so they are testable here."""
    from cfgs import native
    lib = native.load()
    s = native.Settings()
    g = native.Gaussians()
    assert lib.cfgs_preprocess_forward(None, None, None, None, None, None) == 1
    s.image_width = 0
    assert lib.cfgs_preprocess_forward(C.byref(s), C.byref(g), 1, 1, 1, None) == 1
    assert lib.cfgs_render_forward(None, None, None, None, None, 0, None, None, None, None) == 1
    assert lib.cfgs_mark_visible(-1, None, None, None, None, None) == 1
    assert lib.cfgs_pose_grad(5, None, None, None, None, None, None, None, None) == 1
    assert lib.cfgs_pose_adam(1, None, None, None, 1e-3, 0.9, 0.999, 1e-15, None) == 1


def test_dropin_validates_argument_combinations():
    """GaussianRasterizer.forward raises like the upstream module when the SH/colour or
    scale-rotation/covariance choices are not exactly one of each."""
    import torch
    import diff_gaussian_rasterization as dgr
    rs = dgr.GaussianRasterizationSettings(8, 8, 1.0, 1.0, torch.zeros(3), 1.0, torch.eye(4), torch.eye(4), 0,
                                           torch.zeros(3), False, False)
    r = dgr.GaussianRasterizer(rs)
    m = torch.zeros(4, 3)
    o = torch.ones(4, 1)
    with pytest.raises(Exception):
        r(m, m, o, scales=m, rotations=torch.zeros(4, 4))  # neither shs nor colours
    with pytest.raises(Exception):
        r(m, m, o, shs=torch.zeros(4, 1, 3), colors_precomp=m, scales=m, rotations=torch.zeros(4, 4))
    with pytest.raises(Exception):
        r(m, m, o, shs=torch.zeros(4, 1, 3))  # no covariance at all
    with pytest.raises(Exception):
        r(m, m, o, shs=torch.zeros(4, 1, 3), scales=m, rotations=torch.zeros(4, 4), cov3D_precomp=torch.zeros(4, 6))
    with pytest.raises(RuntimeError):  # CPU tensors: no CPU fallback exists
        r(m, m, o, shs=torch.zeros(4, 1, 3), scales=m, rotations=torch.zeros(4, 4))
    assert dgr.GaussianRasterizationSettings._fields == (
        "image_height", "image_width", "tanfovx", "tanfovy", "bg", "scale_modifier", "viewmatrix", "projmatrix",
        "sh_degree", "campos", "prefiltered", "debug")


def test_ssim_abi_host_checks():
    from cfgs import native
    lib = native.load()
    assert lib.cfgs_ssim_scratch_bytes(3, 360, 640) >= 3 * 3 * 360 * 640 * 4
    assert lib.cfgs_ssim_scratch_bytes(0, 10, 10) == 0
    assert lib.cfgs_ssim_forward(3, 0, 10, None, None, None, None, None) == 1
    assert lib.cfgs_ssim_backward(3, 10, 10, None, None, None, None, None, None) == 1


def test_pointcloud_abi_host_checks():
    from cfgs import native
    lib = native.load()
    assert lib.cfgs_pointcloud_workspace_bytes(1000) > 1000 * 16
    assert lib.cfgs_pointcloud_workspace_bytes(-1) == 0
    assert lib.cfgs_depth_to_points(0, 4, None, 1.0, 1.0, 0.0, 0.0, None, None) == 1
    assert lib.cfgs_knn3_mean_dist2(-1, None, None, None, None) == 1
    assert lib.cfgs_knn3_mean_dist2(0, None, None, None, None) == 0
    m = native.C.c_int64(7)
    assert lib.cfgs_voxel_down_sample(10, None, None, 0.0, None, None, None, native.C.byref(m), None) == 1
    assert lib.cfgs_voxel_down_sample(0, None, None, 0.01, None, None, None, native.C.byref(m), None) == 0
    assert m.value == 0


def test_l1_loss_abi_host_checks():
    from cfgs import native
    lib = native.load()
    assert lib.cfgs_l1_loss_scratch_bytes(6_220_800) >= 4 * 152 * 4
    assert lib.cfgs_l1_loss_forward(-1, None, None, 1, None, None, None, None) == 1
    assert lib.cfgs_l1_loss_forward(10, None, None, 1, None, None, None, None) == 1
    assert lib.cfgs_l1_loss_backward(-1, None, None, 0, None, None, None) == 1
    assert lib.cfgs_l1_loss_backward(10, None, None, 0, None, None, None) == 1
    assert lib.cfgs_l1_loss_backward(0, None, None, 0, None, None, None) == 0
