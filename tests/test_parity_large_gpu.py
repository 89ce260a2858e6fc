"""Parity of the benchmarked configurations against the CPU oracle.

The drop-in path at the sizes the benchmark runs: 1,000,000 SH3 Gaussians at 1920x1080
(8,160 tiles, a two-pass tile sort of 13 tile-index bits), 640x360 scenes (920 tiles, two
passes), and a batch of pose solves whose tiles together exceed 2^16 (a three-pass tile
sort). Sort keys, sorted instance order, tile ranges, contributor counts and final
transmittance are compared bit for bit (the outputs scene/gaussian_model_cf.py:873-884
consumes come from them), images within 1e-5 (they are also bit-identical), and every
gradient element within 1e-4 relative of the float64 oracle or, where its terms cancel,
within the float32 rounding bound of the same computation (oracle.error_bound), with no
floor taken from the tensor's largest element. Each tensor's fraction of elements within
1e-4 relative is printed.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import assert_grad_bounded, bits, grad_report, l1_image_grad, settings_for

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def dgr():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as m
    return m


def _scene(case):
    from cfgs import scenes
    if case == "config1_1M_1080p":
        return scenes.scene_large(n=1_000_000, width=1920, height=1080, seed=1)
    if case == "sh3_640x360":
        return scenes.scene_small(n=60_000, width=640, height=360, seed=31)
    if case == "pose_640x360":
        sc = scenes.scene_pose(width=640, height=360, seed=2)
        g = torch.Generator().manual_seed(5)
        sc.target = torch.rand(3, 360, 640, generator=g)
        return sc
    raise ValueError(case)


def _forward_and_backward(dgr, sc):
    """GPU forward (workspaces kept), L1 image gradient plus small depth and alpha
    gradients, GPU backward; the oracle's forward and backward on the same inputs."""
    from cfgs import raster
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds
    rs = settings_for(dgr, sc)
    s = sc.to(DEV)
    color, radii, depth, alpha, state = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales,
                                                       s.rotations, None)
    H, W = sc.camera.height, sc.camera.width
    gen = torch.Generator().manual_seed(7)
    gc = l1_image_grad(color, s.target).contiguous()
    gd = (torch.randn(1, H, W, generator=gen) * 1e-3).to(DEV)
    ga = (torch.randn(1, H, W, generator=gen) * 1e-3).to(DEV)
    grads = raster.backward(rs, state, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None, gc, gd, ga)
    torch.cuda.synchronize()
    views = raster.inspect_state(state, W, H)
    ref = Oracle.from_scene(sc).forward()
    want = ref.backward(gc.cpu().numpy(), gd.cpu().numpy(), ga.cpu().numpy(), magnitudes=True)
    bound = backward_bounds(ref)
    names = ["means2D", "colors", "opacity", "means3D", "cov3D", "sh", "scales", "rotations"]
    got = {k: v.cpu().numpy() for k, v in zip(names, grads)}
    return (color, radii, depth, alpha, state, views), ref, got, want, bound


def _check_forward(out, ref):
    color, radii, depth, alpha, state, v = out
    assert state.num_rendered == ref.K
    np.testing.assert_array_equal(radii.cpu().numpy(), ref.radii)
    vis = ref.radii > 0
    np.testing.assert_array_equal(v["touched"].cpu().numpy().astype(np.uint32), ref.touched)
    np.testing.assert_array_equal(bits(v["rgbd"].cpu().numpy()[vis]), bits(ref.rgbd[vis]))
    np.testing.assert_array_equal(v["tile_range"].cpu().numpy().astype(np.uint32), ref.ranges)
    gid = v["sorted_gid"].cpu().numpy().astype(np.uint32)
    np.testing.assert_array_equal(gid, ref.gid)
    ranges = ref.ranges.astype(np.int64)
    tile_of = np.repeat(np.arange(len(ranges) - 1, dtype=np.uint64), np.diff(ranges))
    keys = (tile_of << np.uint64(32)) | bits(v["rgbd"].cpu().numpy()[gid, 3]).astype(np.uint64)
    np.testing.assert_array_equal(keys, ref.keys)
    np.testing.assert_array_equal(v["n_contrib"].cpu().numpy().astype(np.uint32), ref.n_contrib)
    np.testing.assert_array_equal(bits(v["final_T"].cpu().numpy()), bits(ref.final_T))
    for name, got, want in (("color", color, ref.color), ("depth", depth, ref.depth), ("alpha", alpha, ref.alpha)):
        g = got.cpu().numpy()
        assert np.abs(g - want).max() <= 1e-5, name
        np.testing.assert_array_equal(bits(g), bits(want), err_msg=name)


def _check_gradients(got, want, bound, label):
    for name in got:
        if want.get(name) is None:
            continue
        st = grad_report(got[name], want[name], bound[name])
        print(f"{label} {name}: " + ", ".join(f"{k}={v:.4g}" if isinstance(v, float) else f"{k}={v}"
                                             for k, v in st.items()))
        assert_grad_bounded(f"{label} {name}", got[name], want[name], bound[name])


@pytest.mark.parametrize("case", ["config1_1M_1080p", "sh3_640x360", "pose_640x360"])
def test_benchmarked_sizes_match_oracle(dgr, case):
    sc = _scene(case)
    out, ref, got, want, bound = _forward_and_backward(dgr, sc)
    tiles = ((sc.camera.width + 15) // 16) * ((sc.camera.height + 15) // 16)
    assert tiles > 256  # more than one tile-sort pass of 8 bits
    _check_forward(out, ref)
    _check_gradients(got, want, bound, case)


def _batch_specs():
    """Eight 1920x1080 solves and two 960x540 ones: 69,360 tiles (17 tile-index bits,
    three passes of 6)."""
    specs = [(1920, 1080, 30_000 + 1000 * i, 100 + i) for i in range(8)]
    specs += [(960, 540, 20_000, 200), (960, 540, 45_000, 201)]
    return specs


def test_batched_three_pass_sort_matches_oracle(dgr):
    """One iteration of a batch whose tile count exceeds 2^16: each solve's sorted
    instances, tile ranges, contributor counts, transmittance and image, cut out of the
    batch, equal the oracle's for that solve alone (at the solves' starting pose, the
    identity, where the batched preprocess places every mean exactly as given)."""
    from cfgs import batch, native, pose, scenes
    from oracle.c_oracle import Oracle
    specs = _batch_specs()
    probs, scs = [], []
    for (w, h, n, sd) in specs:
        sc = scenes.scene_pose(width=w, height=h, n=n, seed=sd)
        scs.append(sc)
        probs.append(pose.make_problem(sc, DEV))
    bs = batch.BatchSolver(probs, use_graph=False)
    assert bs.plan.num_tiles > 1 << 16
    args = bs.prepare()
    bs.iterate(args)
    torch.cuda.synchronize()
    T = int(bs.plan.num_tiles)
    il = native.image_layout(16 * T, 16)
    bl = native.binning_layout(bs.capacity)
    img = bs.image
    tile_range = img[il["tile_range"]: il["tile_range"] + 4 * (T + 1)].view(torch.int32).cpu().numpy().astype(np.int64)
    K = int(tile_range[-1])
    sorted_gid = bs.binning[bl["sorted_gid"]: bl["sorted_gid"] + 4 * K].view(torch.int32).cpu().numpy()
    P = int(bs.plan.num_pixels)
    n_contrib = img[il["n_contrib"]: il["n_contrib"] + 4 * P].view(torch.int32).cpu().numpy().astype(np.uint32)
    final_T = img[il["final_T"]: il["final_T"] + 4 * P].view(torch.float32).cpu().numpy()
    color = bs.color.cpu().numpy()
    for s, (sc, p) in enumerate(zip(scs, probs)):
        cam = sc.camera
        ref = Oracle(cam.width, cam.height, cam.tanfovx, cam.tanfovy, sc.bg, 1.0, cam.viewmatrix, cam.projmatrix,
                     sc.sh_degree, cam.campos, sc.means3D, sc.opacities, shs=sc.shs, scales=sc.scales,
                     rotations=sc.rotations).forward()
        tb, gb, pb = int(bs.tile_base[s]), int(bs.gauss_base[s]), int(bs.pix_base[s])
        Ts = ref.gx * ref.gy
        r = tile_range[tb: tb + Ts + 1]
        np.testing.assert_array_equal(r - r[0], ref.ranges.astype(np.int64), err_msg=f"solve {s} ranges")
        np.testing.assert_array_equal(sorted_gid[r[0]: r[-1]] - gb, ref.gid.astype(np.int64), err_msg=f"solve {s}")
        HW = cam.width * cam.height
        np.testing.assert_array_equal(n_contrib[pb: pb + HW], ref.n_contrib, err_msg=f"solve {s} n_contrib")
        np.testing.assert_array_equal(bits(final_T[pb: pb + HW]), bits(ref.final_T), err_msg=f"solve {s} final_T")
        np.testing.assert_array_equal(bits(color[3 * pb: 3 * pb + 3 * HW]), bits(ref.color.reshape(-1)),
                                      err_msg=f"solve {s} colour")
