"""GPU parity of the rasteriser against the CPU oracle (bit-exact forward integer and
float outputs, gradients within 1e-4 relative) and against torch float64 autograd."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import assert_grad_bounded, bits, l1_image_grad, settings_for

pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def dgr():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as m
    return m


def _oracle(scene, **kw):
    from oracle.c_oracle import Oracle
    return Oracle.from_scene(scene, **kw).forward()


def _gpu_forward(dgr, scene, **kw):
    from cfgs import raster
    rs = settings_for(dgr, scene, **kw)
    s = scene.to(DEV)
    color, radii, depth, alpha, state = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales,
                                                       s.rotations, None)
    torch.cuda.synchronize()
    views = raster.inspect_state(state, scene.camera.width, scene.camera.height)
    return color, radii, depth, alpha, state, views


def _dense_scene(n=9000, seed=21):
    """Many Gaussians inside a few tiles: exercises the tile sort's merge path (> 4096
    instances in a tile) plus a few screen-filling Gaussians."""
    from cfgs import scenes
    sc = scenes.scene_small(n=n, width=64, height=48, seed=seed)
    rng = np.random.default_rng(seed)
    m = sc.means3D.numpy().copy()
    z = rng.uniform(2.0, 6.0, n)
    m[:, 0] = rng.uniform(-0.12, 0.12, n) * z
    m[:, 1] = rng.uniform(-0.12, 0.12, n) * z
    m[:, 2] = z
    s = sc.scales.numpy().copy()
    s[:5] = 0.6  # a few Gaussians that cover every tile
    sc.means3D = torch.from_numpy(m.astype(np.float32))
    sc.scales = torch.from_numpy(s.astype(np.float32))
    return sc


def _check_forward_bits(scene, out, ref):
    color, radii, depth, alpha, state, v = out
    assert state.num_rendered == ref.K
    np.testing.assert_array_equal(radii.cpu().numpy(), ref.radii)
    vis = ref.radii > 0
    np.testing.assert_array_equal(v["touched"].cpu().numpy().astype(np.uint32), ref.touched)
    np.testing.assert_array_equal(bits(v["xy"].cpu().numpy()[vis]), bits(ref.xy[vis]))
    np.testing.assert_array_equal(bits(v["conic_op"].cpu().numpy()[vis]), bits(ref.conic_op[vis]))
    np.testing.assert_array_equal(bits(v["rgbd"].cpu().numpy()[vis]), bits(ref.rgbd[vis]))
    np.testing.assert_array_equal(v["tile_range"].cpu().numpy().astype(np.uint32), ref.ranges)
    gid = v["sorted_gid"].cpu().numpy().astype(np.uint32)
    np.testing.assert_array_equal(gid, ref.gid)
    # the 64-bit keys upstream sorts: tile << 32 | depth bits
    ranges = ref.ranges.astype(np.int64)
    tile_of = np.repeat(np.arange(len(ranges) - 1, dtype=np.uint64), np.diff(ranges))
    depth_bits = bits(v["rgbd"].cpu().numpy()[gid, 3]).astype(np.uint64)
    keys = (tile_of << np.uint64(32)) | depth_bits
    np.testing.assert_array_equal(keys, ref.keys)
    np.testing.assert_array_equal(v["n_contrib"].cpu().numpy().astype(np.uint32), ref.n_contrib)
    np.testing.assert_array_equal(bits(v["final_T"].cpu().numpy()), bits(ref.final_T))
    # images: tolerance 1e-5 max-abs; the kernels reproduce the oracle's rounding, so
    # they are expected to be bit-identical as well
    for name, got, want in (("color", color, ref.color), ("depth", depth, ref.depth), ("alpha", alpha, ref.alpha)):
        g = got.cpu().numpy()
        assert np.abs(g - want).max() <= 1e-5, name
        np.testing.assert_array_equal(bits(g), bits(want), err_msg=name)


@pytest.mark.parametrize("case", ["config0", "odd_size", "dense_tiles"])
def test_forward_bit_exact(dgr, case):
    from cfgs import scenes
    if case == "config0":
        sc = scenes.scene_small(n=16384, width=256, height=256, seed=0)
    elif case == "odd_size":
        sc = scenes.scene_small(n=2500, width=100, height=75, seed=7)
    else:
        sc = _dense_scene()
    out = _gpu_forward(dgr, sc)
    ref = _oracle(sc)
    if case == "dense_tiles":
        assert int(np.diff(ref.ranges.astype(np.int64)).max()) > 4096
    _check_forward_bits(sc, out, ref)


def _run_autograd(dgr, scene, gd_seed=0, use_colors=False, use_cov=False, colors=None, cov=None):
    rs = settings_for(dgr, scene)
    s = scene.to(DEV)
    leaves = {"means3D": s.means3D.clone().requires_grad_(True),
              "means2D": torch.zeros_like(s.means3D, requires_grad=True),
              "opacities": s.opacities.clone().requires_grad_(True)}
    kw = {}
    if use_colors:
        leaves["colors_precomp"] = colors.to(DEV).clone().requires_grad_(True)
        kw["colors_precomp"] = leaves["colors_precomp"]
    else:
        leaves["shs"] = s.shs.clone().requires_grad_(True)
        kw["shs"] = leaves["shs"]
    if use_cov:
        leaves["cov3D_precomp"] = cov.to(DEV).clone().requires_grad_(True)
        kw["cov3D_precomp"] = leaves["cov3D_precomp"]
    else:
        leaves["scales"] = s.scales.clone().requires_grad_(True)
        leaves["rotations"] = s.rotations.clone().requires_grad_(True)
        kw["scales"] = leaves["scales"]
        kw["rotations"] = leaves["rotations"]
    color, radii, depth, alpha = dgr.GaussianRasterizer(rs)(means3D=leaves["means3D"], means2D=leaves["means2D"],
                                                            opacities=leaves["opacities"], **kw)
    g = torch.Generator().manual_seed(gd_seed)
    H, W = scene.camera.height, scene.camera.width
    gc = l1_image_grad(color, s.target) if s.target is not None else torch.randn(3, H, W, generator=g).to(DEV)
    gdep = (torch.randn(1, H, W, generator=g) * 1e-3).to(DEV)
    galp = (torch.randn(1, H, W, generator=g) * 1e-3).to(DEV)
    torch.autograd.backward([color, depth, alpha], [gc, gdep, galp])
    torch.cuda.synchronize()
    return color, radii, depth, alpha, leaves, (gc.cpu(), gdep.cpu(), galp.cpu())


@pytest.mark.parametrize("case", ["config0", "odd_size", "dense_tiles"])
def test_backward_matches_oracle(dgr, case):
    from cfgs import scenes
    if case == "config0":
        sc = scenes.scene_small(n=16384, width=256, height=256, seed=0)
    elif case == "odd_size":
        sc = scenes.scene_small(n=2500, width=100, height=75, seed=7)
    else:
        sc = _dense_scene()
    color, radii, depth, alpha, leaves, (gc, gd, ga) = _run_autograd(dgr, sc)
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds
    ref = Oracle.from_scene(sc).forward()
    want = ref.backward(gc.numpy(), gd.numpy(), ga.numpy(), magnitudes=True)
    bound = backward_bounds(ref)
    for leaf, key in (("means2D", "means2D"), ("opacities", "opacity"), ("means3D", "means3D"), ("shs", "sh"),
                      ("scales", "scales"), ("rotations", "rotations")):
        assert_grad_bounded(leaf, leaves[leaf].grad.cpu(), want[key], bound[key])


def test_backward_matches_torch_autograd(dgr):
    """Independent check of the hand-derived backward: float64 autograd of the dense
    torch restatement (its own decisions, its own derivatives)."""
    from cfgs import scenes
    from oracle import torch_oracle as TO
    sc = scenes.scene_small(n=500, width=80, height=64, seed=3)
    color, radii, depth, alpha, leaves, (gc, gd, ga) = _run_autograd(dgr, sc, gd_seed=4)
    cam = sc.camera
    ref = {k: getattr(sc, k).double().clone().requires_grad_(True)
           for k in ["means3D", "opacities", "shs", "scales", "rotations"]}
    m2 = torch.zeros(sc.n, 3, dtype=torch.float64, requires_grad=True)
    r = TO.rasterize(cam.width, cam.height, cam.tanfovx, cam.tanfovy, sc.bg, 1.0, cam.viewmatrix, cam.projmatrix,
                     sc.sh_degree, cam.campos, ref["means3D"], m2, ref["opacities"], shs=ref["shs"],
                     scales=ref["scales"], rotations=ref["rotations"])
    assert np.abs(r["color"].detach().numpy() - color.detach().cpu().numpy()).max() <= 1e-5
    np.testing.assert_array_equal(r["radii"].numpy(), radii.cpu().numpy())
    L = (r["color"] * gc.double()).sum() + (r["depth"] * gd.double()).sum() + (r["alpha"] * ga.double()).sum()
    L.backward()
    # the float32 rounding bound of the kernels' computation on this scene (the dense
    # float64 restatement is exact to far below it)
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds
    co = Oracle.from_scene(sc).forward()
    co.backward(gc.numpy(), gd.numpy(), ga.numpy(), magnitudes=True)
    bound = backward_bounds(co)
    assert_grad_bounded("means2D", leaves["means2D"].grad.cpu(), m2.grad, bound["means2D"])
    assert_grad_bounded("means3D", leaves["means3D"].grad.cpu(), ref["means3D"].grad, bound["means3D"])
    assert_grad_bounded("opacities", leaves["opacities"].grad.cpu(), ref["opacities"].grad, bound["opacity"])
    assert_grad_bounded("shs", leaves["shs"].grad.cpu(), ref["shs"].grad, bound["sh"])
    assert_grad_bounded("scales", leaves["scales"].grad.cpu(), ref["scales"].grad, bound["scales"])
    assert_grad_bounded("rotations", leaves["rotations"].grad.cpu(), ref["rotations"].grad, bound["rotations"])


def test_precomputed_inputs_match(dgr):
    """The reference's own switches (scene/gaussian_model_cf.py:834-866): SH colours
    computed in Python (+0.5, clamp at 0) and covariances from build_scaling_rotation
    give the same image as the in-kernel paths."""
    from cfgs import scenes
    from oracle import torch_oracle as TO
    sc = scenes.scene_small(n=3000, width=128, height=96, seed=9)
    rs = settings_for(dgr, sc)
    s = sc.to(DEV)
    m2 = torch.zeros_like(s.means3D)
    base, _, _, _ = dgr.GaussianRasterizer(rs)(means3D=s.means3D, means2D=m2, opacities=s.opacities, shs=s.shs,
                                               scales=s.scales, rotations=s.rotations)
    d = s.means3D - s.camera.campos[None]
    d = d / d.norm(dim=1, keepdim=True)
    B = TO.sh_basis(3, d.double().cpu()).float().to(DEV)
    colors = torch.clamp_min((B[:, :, None] * s.shs).sum(1) + 0.5, 0.0)
    cov = TO.cov3d(s.scales.double().cpu(), s.rotations.double().cpu(), 1.0).float().to(DEV)
    img_c, _, _, _ = dgr.GaussianRasterizer(rs)(means3D=s.means3D, means2D=m2, opacities=s.opacities,
                                                colors_precomp=colors, scales=s.scales, rotations=s.rotations)
    img_v, _, _, _ = dgr.GaussianRasterizer(rs)(means3D=s.means3D, means2D=m2, opacities=s.opacities, shs=s.shs,
                                                cov3D_precomp=cov)
    assert (img_c - base).abs().max().item() <= 1e-5
    assert (img_v - base).abs().max().item() <= 1e-4


def test_precomputed_backward_matches_oracle(dgr):
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    sc = scenes.scene_small(n=2000, width=96, height=80, seed=12)
    g = torch.Generator().manual_seed(1)
    colors = torch.rand(sc.n, 3, generator=g)
    from oracle import torch_oracle as TO
    cov = TO.cov3d(sc.scales.double(), sc.rotations.double(), 1.0).float()
    sc.target = torch.rand(3, sc.camera.height, sc.camera.width, generator=g)
    color, radii, depth, alpha, leaves, (gc, gd, ga) = _run_autograd(dgr, sc, use_colors=True, use_cov=True,
                                                                     colors=colors, cov=cov)
    ref = Oracle.from_scene(sc, use_colors=True, colors=colors, use_cov=True, cov=cov).forward()
    np.testing.assert_array_equal(bits(color.detach().cpu().numpy()), bits(ref.color))
    want = ref.backward(gc.numpy(), gd.numpy(), ga.numpy(), magnitudes=True)
    from oracle.error_bound import backward_bounds
    bound = backward_bounds(ref)
    assert_grad_bounded("colors_precomp", leaves["colors_precomp"].grad.cpu(), want["colors"], bound["colors"])
    assert_grad_bounded("cov3D_precomp", leaves["cov3D_precomp"].grad.cpu(), want["cov3D"], bound["cov3D"])
    assert_grad_bounded("means3D", leaves["means3D"].grad.cpu(), want["means3D"], bound["means3D"])


def test_empty_and_culled(dgr):
    from cfgs import scenes
    sc = scenes.scene_small(n=64, width=48, height=40, seed=1)
    sc.bg = torch.tensor([0.25, 0.5, 0.75])
    sc.means3D[:, 2] = 0.1  # every Gaussian behind the near plane
    color, radii, depth, alpha, leaves, _ = _run_autograd(dgr, sc)
    assert int(radii.abs().sum()) == 0
    assert torch.equal(color.detach().cpu(), sc.bg[:, None, None].expand(3, 40, 48).contiguous())
    assert float(alpha.detach().abs().max()) == 0.0
    assert float(leaves["means3D"].grad.abs().max()) == 0.0
    empty = scenes.scene_small(n=0, width=33, height=17, seed=1)
    color, radii, depth, alpha, state, v = _gpu_forward(dgr, empty)
    assert state.num_rendered == 0 and radii.numel() == 0
    assert float(color.abs().max()) == 0.0


def test_prefiltered_violation_raises(dgr):
    from cfgs import scenes
    sc = scenes.scene_small(n=32, width=32, height=32, seed=2)
    sc.means3D[0, 2] = 0.05
    with pytest.raises(RuntimeError):
        _gpu_forward(dgr, sc, prefiltered=True)


def test_deterministic(dgr):
    from cfgs import scenes
    sc = scenes.scene_small(n=8000, width=128, height=128, seed=5)
    a = _run_autograd(dgr, sc)
    b = _run_autograd(dgr, sc)
    assert torch.equal(a[0], b[0])
    for k in a[4]:
        assert torch.equal(a[4][k].grad, b[4][k].grad), k


def test_mark_visible(dgr):
    from cfgs import scenes
    sc = scenes.scene_small(n=1000, width=64, height=64, seed=4)
    sc.means3D[::3, 2] = 0.15
    rs = settings_for(dgr, sc)
    vis = dgr.GaussianRasterizer(rs).markVisible(sc.means3D.to(DEV)).cpu()
    t = torch.cat([sc.means3D, torch.ones(sc.n, 1)], 1) @ sc.camera.viewmatrix[:, 2]
    assert torch.equal(vis, t > 0.2)


def test_unused_outputs_give_same_gradients(dgr):
    """A loss on the colour alone: autograd hands the backward no depth / alpha gradients
    (None instead of zeros), which must give the same gradient bits as explicit zeros."""
    from cfgs import raster, scenes
    sc = scenes.scene_small(n=3000, width=96, height=80, seed=17)
    rs = settings_for(dgr, sc)
    s = sc.to(DEV)
    leaves = [t.clone().requires_grad_(True) for t in (s.means3D, s.opacities, s.shs, s.scales, s.rotations)]
    m2 = torch.zeros_like(s.means3D, requires_grad=True)
    color, radii, depth, alpha = dgr.GaussianRasterizer(rs)(means3D=leaves[0], means2D=m2, opacities=leaves[1],
                                                            shs=leaves[2], scales=leaves[3], rotations=leaves[4])
    g = l1_image_grad(color, s.target)
    color.backward(g)
    c2, r2, d2, a2, st = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
    z = torch.zeros_like(d2)
    d_m2, d_col, d_op, d_m3, d_cov, d_sh, d_sc, d_rot = raster.backward(
        rs, st, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None, g, z, z)
    for got, want in [(leaves[0].grad, d_m3), (leaves[1].grad, d_op), (leaves[2].grad, d_sh), (leaves[3].grad, d_sc),
                      (leaves[4].grad, d_rot), (m2.grad, d_m2)]:
        assert torch.equal(got, want)


def test_split_binning_equals_one_call(dgr):
    """cfgs_depth_order + cfgs_bin_instances (the drop-in forward's split, which lets the
    depth sort run while the host reads K) leave the same workspaces as cfgs_bin_forward."""
    import ctypes as C
    from cfgs import native, raster, scenes
    sc = scenes.scene_small(n=5000, width=160, height=120, seed=23)
    rs = settings_for(dgr, sc)
    s = sc.to(DEV)
    color, radii, depth, alpha, st = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations,
                                                    None)
    ref = raster.inspect_state(st, sc.camera.width, sc.camera.height)
    lib = native.load()
    keep: list = []
    cs = raster.make_settings(rs, keep)
    g = raster.make_gaussians(s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
    binning = torch.zeros_like(st.binning)
    native.check(lib.cfgs_bin_forward(C.byref(cs), C.byref(g), st.geom.data_ptr(), st.image.data_ptr(),
                                      binning.data_ptr(), st.num_rendered, raster.stream_handle(s.means3D.device)),
                 "cfgs_bin_forward")
    torch.cuda.synchronize()
    got = raster.inspect_state(raster.ForwardState(st.geom, st.image, binning, st.num_rendered, st.radii),
                               sc.camera.width, sc.camera.height)
    for k in ("sorted_gid", "sorted_pidx", "tile_range", "offset"):
        assert torch.equal(got[k], ref[k]), k


SETTING_CASES = {
    "white_background": dict(bg=(1.0, 1.0, 1.0), scale=1.0, degree=None),
    "colour_background_scaled": dict(bg=(0.2, 0.5, 0.8), scale=0.7, degree=None),
    "sh_degree_1_of_3": dict(bg=None, scale=1.0, degree=1),
    "sh_degree_2_of_3_scaled": dict(bg=(0.3, 0.3, 0.3), scale=1.3, degree=2),
}


@pytest.mark.parametrize("case", list(SETTING_CASES))
def test_settings_variants_match_oracle(dgr, case):
    """The settings the reference varies across training: a white or coloured background
    (`white_background`), scale_modifier, and an active SH degree below the stored
    coefficients (the degree rises during training, scene/gaussian_model_cf.py
    oneupSHdegree). Forward outputs bit-exact, gradients within 1e-4 relative or the
    float32 bound."""
    from cfgs import scenes
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds
    c = SETTING_CASES[case]
    sc = scenes.scene_small(n=3000, width=96, height=80, seed=13)
    if c["bg"] is not None:
        sc.bg = torch.tensor(c["bg"], dtype=torch.float32)
    if c["degree"] is not None:
        sc.sh_degree = c["degree"]
    rs = settings_for(dgr, sc, scale_modifier=c["scale"])
    s = sc.to(DEV)
    leaves = {"means3D": s.means3D.clone().requires_grad_(True),
              "means2D": torch.zeros_like(s.means3D, requires_grad=True),
              "opacities": s.opacities.clone().requires_grad_(True), "shs": s.shs.clone().requires_grad_(True),
              "scales": s.scales.clone().requires_grad_(True), "rotations": s.rotations.clone().requires_grad_(True)}
    color, radii, depth, alpha = dgr.GaussianRasterizer(rs)(**leaves)
    H, W = sc.camera.height, sc.camera.width
    g = torch.Generator().manual_seed(3)
    gc, gd, ga = torch.randn(3, H, W, generator=g), torch.randn(1, H, W, generator=g), torch.randn(1, H, W, generator=g)
    torch.autograd.backward([color, depth, alpha], [gc.to(DEV), gd.to(DEV), ga.to(DEV)])
    torch.cuda.synchronize()
    ref = Oracle.from_scene(sc, scale_modifier=c["scale"]).forward()
    np.testing.assert_array_equal(radii.cpu().numpy(), ref.radii)
    for got, want in ((color, ref.color), (depth, ref.depth), (alpha, ref.alpha)):
        np.testing.assert_array_equal(bits(got.detach().cpu().numpy()), bits(want))
    want = ref.backward(gc.numpy(), gd.numpy(), ga.numpy(), magnitudes=True)
    bound = backward_bounds(ref)
    for leaf, key in (("means2D", "means2D"), ("opacities", "opacity"), ("means3D", "means3D"), ("shs", "sh"),
                      ("scales", "scales"), ("rotations", "rotations")):
        assert_grad_bounded(leaf, leaves[leaf].grad.cpu(), want[key], bound[key])
