"""The plain GPU path (include/cfgs_plain.h: 64-bit keys and one radix sort, one thread
per pixel, global atomic gradients) against the oracle and the tuned path.

It shares the per-pixel arithmetic with the tuned kernels, so its forward must equal
the oracle bit for bit (colour, depth, alpha, radii, contributor counts, final
transmittance). Its gradients are sums formed by atomic adds in whatever order the
threads arrive, so they are held to 1e-4 relative or the float32 bound of a sum of that
many terms in any order (oracle.error_bound with the contribution counts).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import assert_grad_bounded, bits, settings_for

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
    if case == "config0":
        return scenes.scene_small(n=16384, width=256, height=256, seed=0)
    if case == "odd_size":
        return scenes.scene_small(n=2500, width=100, height=75, seed=7)
    return scenes.scene_small(n=6000, width=640, height=360, seed=11)  # 920 tiles: 11 tile bits


def _plain_forward(dgr, sc, capacity_hint=1):
    from cfgs import native, plain
    rs = settings_for(dgr, sc)
    s = sc.to(DEV)
    out = plain.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None,
                        capacity_hint=capacity_hint)
    torch.cuda.synchronize()
    st = out[4]
    il = native.image_layout(sc.camera.width, sc.camera.height)
    HW = sc.camera.width * sc.camera.height
    final_T = st.image[il["final_T"]: il["final_T"] + 4 * HW].view(torch.float32)
    n_contrib = st.image[il["n_contrib"]: il["n_contrib"] + 4 * HW].view(torch.int32)
    return rs, s, out, final_T, n_contrib


@pytest.mark.parametrize("case", ["config0", "odd_size", "wide"])
def test_plain_forward_bit_exact(dgr, case):
    from oracle.c_oracle import Oracle
    sc = _scene(case)
    _, _, (color, radii, depth, alpha, st), final_T, n_contrib = _plain_forward(dgr, sc)
    ref = Oracle.from_scene(sc).forward()
    assert st.num_rendered == ref.K and st.capacity == ref.K  # grown from a capacity of 1
    np.testing.assert_array_equal(radii.cpu().numpy(), ref.radii)
    np.testing.assert_array_equal(n_contrib.cpu().numpy().astype(np.uint32), ref.n_contrib)
    np.testing.assert_array_equal(bits(final_T.cpu().numpy()), bits(ref.final_T))
    np.testing.assert_array_equal(bits(color.cpu().numpy()), bits(ref.color))
    np.testing.assert_array_equal(bits(depth.cpu().numpy()), bits(ref.depth))
    np.testing.assert_array_equal(bits(alpha.cpu().numpy()), bits(ref.alpha))


def test_plain_forward_equals_tuned_path(dgr):
    from cfgs import raster
    sc = _scene("config0")
    rs, s, (color, radii, depth, alpha, _), _, _ = _plain_forward(dgr, sc, capacity_hint=1 << 20)
    c2, r2, d2, a2, _ = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
    assert torch.equal(radii, r2)
    for x, y in ((color, c2), (depth, d2), (alpha, a2)):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))


@pytest.mark.parametrize("case", ["config0", "odd_size"])
def test_plain_backward_matches_oracle(dgr, case):
    from cfgs import plain
    from oracle.c_oracle import Oracle
    from oracle.error_bound import backward_bounds, contribution_counts
    sc = _scene(case)
    rs, s, (color, radii, depth, alpha, st), _, _ = _plain_forward(dgr, sc)
    H, W = sc.camera.height, sc.camera.width
    g = torch.Generator().manual_seed(5)
    gc, gd, ga = torch.randn(3, H, W, generator=g), torch.randn(1, H, W, generator=g), torch.randn(1, H, W, generator=g)
    grads = plain.backward(rs, st, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None,
                           gc.to(DEV), gd.to(DEV), ga.to(DEV))
    torch.cuda.synchronize()
    ref = Oracle.from_scene(sc).forward()
    want = ref.backward(gc.numpy(), gd.numpy(), ga.numpy(), magnitudes=True)
    bound = backward_bounds(ref, terms=contribution_counts(ref))
    names = ("means2D", "colors", "opacity", "means3D", "cov3D", "sh", "scales", "rotations")
    for name, got in zip(names, grads):
        assert_grad_bounded(name, got.cpu(), want[name], bound[name])


def test_plain_forward_equals_tuned_path_at_1080p(dgr):
    """The benchmarked workload (1M SH-degree-3 Gaussians, 1920x1080, 8160 tiles: 13 tile
    bits in the plain path's 45-bit keys): the plain forward equals the tuned path's
    bit for bit, so the two timings are of the same result."""
    from cfgs import raster, scenes
    sc = scenes.scene_large(n=1_000_000, width=1920, height=1080, seed=1)
    rs, s, (color, radii, depth, alpha, st), final_T, n_contrib = _plain_forward(dgr, sc, capacity_hint=1 << 24)
    c2, r2, d2, a2, st2 = raster.forward(rs, s.means3D, s.opacities, s.shs, None, s.scales, s.rotations, None)
    v = raster.inspect_state(st2, 1920, 1080)
    assert st.num_rendered == st2.num_rendered
    assert torch.equal(radii, r2)
    assert torch.equal(n_contrib, v["n_contrib"])
    assert torch.equal(final_T.view(torch.int32), v["final_T"].view(torch.int32))
    for x, y in ((color, c2), (depth, d2), (alpha, a2)):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))
