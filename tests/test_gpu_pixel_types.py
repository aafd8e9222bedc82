"""The reference's other pixel pipelines: uchar3 (RGB, no alpha), float4 and float3
(CudaStitchPano*<uchar3, float3>, <float4, float4>, <float3, float3>), run by the level-by-level
kernels of hmp_generic.cu.

- uchar3 against the oracle's 3-channel restatement (pinned to the reference's Python port by the
  RGB golden cases, which test_gpu_parity.py also runs on the GPU), every stitcher kind;
- float pipelines against the uint8 ones on the same frames: outside the write rect the canvas is
  the same copy, inside it the float reconstruction packs to the uint8 canvas bit for bit (the
  arithmetic before the pack is the same); float4 against the fused RGBA8 path.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu

RIGS = [
    # (workload, kind, scale, extra rig kwargs)
    ("pano2_1280x720_to_2200x800", 2, 0.5, {"oob_fraction": 0.02}),
    ("pano3_2704x1520_to_6000x1800", 3, 0.25, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 0.25, {}),
]


def _run(st, frames_np, dtype):
    import torch

    ins = [torch.from_numpy(np.ascontiguousarray(f)).cuda().to(dtype) for f in frames_np]
    out = st._run(ins)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _pack(v: np.ndarray) -> np.ndarray:
    return np.where(v <= 0, 0, np.where(v >= 255, 255, np.trunc(np.clip(v, 0, 255)))).astype(np.uint8)


@pytest.mark.parametrize("levels", [0, 3, 6])
@pytest.mark.parametrize("rig_spec", RIGS, ids=[r[0] for r in RIGS])
def test_rgb_matches_oracle(oracle_lib, rig_spec, levels):
    import torch
    from hmpano import synth

    workload, kind, scale, rkw = rig_spec
    rig = synth.workload_rig(workload, seed=41, kind=kind, scale=scale, **rkw)
    frames = [f[..., :3].copy() for f in synth.rig_frames(rig, seed=8, batch=2)]
    st = make_stitcher(kind, masks_for_rig(rig), levels, 2)
    out = _run(st, frames, torch.uint8)
    ref = oracle_lib.Stitch.from_rig(rig, levels, 2).run(frames)
    assert out.shape == ref.shape
    if not np.array_equal(out, ref):
        d = np.abs(out.astype(int) - ref.astype(int))
        pytest.fail(f"uchar3 differs from the oracle: max {d.max()}, pixels {np.argwhere(d.max(-1) > 0)[:4].tolist()}")


@pytest.mark.parametrize("channels", [4, 3])
@pytest.mark.parametrize("levels", [0, 4])
@pytest.mark.parametrize("rig_spec", RIGS, ids=[r[0] for r in RIGS])
def test_float_pipelines_pack_to_uint8(rig_spec, levels, channels):
    import torch
    from hmpano import synth

    workload, kind, scale, rkw = rig_spec
    rig = synth.workload_rig(workload, seed=43, kind=kind, scale=scale, **rkw)
    frames = [f[..., :channels].copy() for f in synth.rig_frames(rig, seed=9, batch=2)]
    st = make_stitcher(kind, masks_for_rig(rig), levels, 2)
    u8 = _run(st, frames, torch.uint8)
    f32 = _run(st, frames, torch.float32)
    assert f32.dtype == np.float32 and f32.shape == u8.shape
    np.testing.assert_array_equal(_pack(f32), u8)
    info = st.info()
    wx, wy, ww, wh = info["write_rect"]
    outside = np.ones(u8.shape[1:3], bool)
    if levels:
        outside[wy:wy + wh, wx:wx + ww] = False
    np.testing.assert_array_equal(f32[:, outside], u8[:, outside].astype(np.float32))


def test_pipeline_errors():
    import torch
    from hmpano import pano, synth

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=3, kind=2, scale=0.25)
    frames = synth.rig_frames(rig, seed=1, batch=1)
    f16 = make_stitcher(2, masks_for_rig(rig), 3, 1, storage="f16")
    with pytest.raises(pano.CudaStatusError, match="RGBA8-only"):
        _run(f16, [f[..., :3].copy() for f in frames], torch.uint8)
    st = make_stitcher(2, masks_for_rig(rig), 3, 1)
    mixed = [torch.from_numpy(frames[0][..., :3].copy()).cuda(), torch.from_numpy(frames[1]).cuda()]
    with pytest.raises(ValueError, match="one pixel type"):
        st._run(mixed)
