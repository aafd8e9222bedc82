"""The reference's N-image stitcher tests (src/pano/cudaPanoN_test.cpp:192-298) on the GPU:
CudaStitchPanoN on identity remaps and pattern frames, with and without the minimised blend.

- uint8 frames: every canvas equals the oracle's bit for bit, so minimised == full as there;
- float4 frames (the reference runs these tests on CudaStitchPanoN<float4, float4>): minimised
  and full canvases agree within the reference's 1e-4, pack to the uint8 canvas, and an uncovered
  gap keeps alpha 0.
"""
from __future__ import annotations

import numpy as np
import pytest

import pano_layouts as pl
from helpers import masks_for

pytestmark = pytest.mark.gpu

TOL = 1e-4  # the reference's kTol for these tests


def _run(lay, minimize, dtype):
    import torch

    import hmpano

    mx, my = pl.tables(lay)
    px, py = zip(*lay["positions"])
    masks = masks_for(pl.KIND_PANON, mx, my, px, py, lay["seam"])
    st = hmpano.CudaStitchPanoN(1, lay["levels"], masks, quiet=True, minimize_blend=minimize)
    ins = [torch.from_numpy(np.ascontiguousarray(f)).cuda().to(dtype) for f in pl.frames(lay)]
    out = st.process(ins)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", ["two_way_overlap", "no_overlap", "gap", "multi_seam_intersection"])
def test_layout_uint8_matches_oracle(oracle_lib, name):
    import torch

    lay = pl.layouts()[name]
    mx, my = pl.tables(lay)
    px, py = zip(*lay["positions"])
    for minimize in (False, True):
        ref = oracle_lib.Stitch(pl.KIND_PANON, mx, my, px, py, lay["seam"], lay["levels"], 1, minimize).run(
            pl.frames(lay))
        out = _run(lay, minimize, torch.uint8)
        assert np.array_equal(out, ref), (name, minimize, int(np.abs(out.astype(int) - ref.astype(int)).max()))


@pytest.mark.parametrize("name", ["two_way_overlap", "no_overlap", "gap", "multi_seam_intersection"])
def test_layout_float4_minimized_equals_full(name):
    import torch

    lay = pl.layouts()[name]
    full = _run(lay, False, torch.float32)
    mini = _run(lay, True, torch.float32)
    assert full.dtype == np.float32 and full.shape == mini.shape
    np.testing.assert_allclose(mini, full, atol=TOL, rtol=0)
    u8 = _run(lay, True, torch.uint8)
    packed = np.where(mini <= 0, 0, np.where(mini >= 255, 255, np.trunc(np.clip(mini, 0, 255)))).astype(np.uint8)
    np.testing.assert_array_equal(packed, u8)
    if lay["gap"]:
        x0, x1 = lay["gap"]
        assert (mini[0, :, x0:x1, 3] == 0).all()
