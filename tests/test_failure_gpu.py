"""Failure detection on the GPU without a GPU fault: a bounded device wait that runs out
returns an error status the host reads, and the context stays usable afterwards.

The library's kernels wait for their bulk/tensor copies on an mbarrier with a bounded
number of polls. cfgs_diag_copy_timeout arms an mbarrier that no copy completes and
runs that same wait with a short limit; the wait gives up, the kernel raises
CFGS_FLAG_COPY_TIMEOUT and returns, and the call returns CFGS_ERR_DEVICE_FLAG. A normal
render on the same device then still matches the oracle bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from helpers import bits, settings_for

pytestmark = pytest.mark.gpu
DEVICE_FLAG, COPY_TIMEOUT = 4, 0x4


def test_bounded_copy_wait_runs_out_and_reports():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import diff_gaussian_rasterization as dgr
    from cfgs import native, raster, scenes
    from oracle.c_oracle import Oracle
    lib = native.load()
    flags = torch.full((1,), 0xFFFF, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for polls in (1, 64, 4096):
        rc = lib.cfgs_diag_copy_timeout(polls, flags.data_ptr(), stream)
        assert rc == DEVICE_FLAG, (polls, rc)
        assert int(flags.item()) == COPY_TIMEOUT
    assert lib.cfgs_diag_copy_timeout(0, flags.data_ptr(), stream) == 1
    assert lib.cfgs_diag_copy_timeout(1 << 23, flags.data_ptr(), stream) == 1
    # the context is still usable: a render afterwards is exact
    sc = scenes.scene_small(n=2000, width=96, height=64, seed=4)
    s = sc.to("cuda")
    color, radii, depth, alpha, st = raster.forward(settings_for(dgr, sc), s.means3D, s.opacities, s.shs, None,
                                                    s.scales, s.rotations, None)
    torch.cuda.synchronize()
    ref = Oracle.from_scene(sc).forward()
    np.testing.assert_array_equal(bits(color.cpu().numpy()), bits(ref.color))
