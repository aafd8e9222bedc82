"""GPU parity at the full sizes of the named workloads, through the C ABI, against the oracle.

* eight images 8 x 2000x1500 -> 9000x2400 (45-degree yaw steps), 6 levels, N-way rule;
* the three-image stream of the batched workload, 3 x 2704x1520 -> 6000x1800, 6 levels;
* the two-image production frame 2 x 5120x2880 -> 8500x3300 with the 5-tap Binomial5 filter.

FP32 storage must equal the FP32 oracle bit for bit; FP16 level storage must stay within 1 uint8
LSB (max) and 0.05 LSB (mean) of the FP64 oracle. The hard seam of the same rigs is bit-exact.
At these sizes tiles meet the planes' edges, the seams and the blend region's borders in every
combination, and the per-tile slot lists reach their largest lengths.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_stitch, lsb_stats, make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu

F16_MAX_LSB = 1
F16_MEAN_LSB = 0.05


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _full_scale(oracle_lib, workload, kind, levels=6, filt="refbox"):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=1234, kind=kind)
    frames = synth.rig_frames(rig, seed=3)
    fid = oracle_lib.FILTER_BINOMIAL5 if filt == "binomial5" else oracle_lib.FILTER_REFBOX
    o = oracle_lib.Stitch.from_rig(rig, levels, filter=fid)
    st = make_stitcher(kind, masks_for_rig(rig), levels, filter=filt)
    assert st.status.ok(), st.status
    out = gpu_stitch(st, frames)
    ref = o.run(frames)
    if not np.array_equal(out, ref):
        mx, mean = lsb_stats(out, ref)
        bad = np.argwhere(np.abs(out.astype(int) - ref.astype(int)).max(-1) > 0)
        pytest.fail(f"{workload} FP32 differs from the FP32 oracle: max {mx} LSB, mean {mean:.6f}, "
                    f"{len(bad)} pixels, first {bad[:5].tolist()}")
    st16 = make_stitcher(kind, masks_for_rig(rig), levels, filter=filt, storage="f16")
    out16 = gpu_stitch(st16, frames)
    mx, mean = lsb_stats(out16, o.run(frames, "f64"))
    assert mx <= F16_MAX_LSB and mean <= F16_MEAN_LSB, (workload, "f16", mx, mean)
    return rig, frames


def test_eight_images_9000x2400_l6(oracle_lib):
    rig, frames = _full_scale(oracle_lib, "panon8_2000x1500_to_9000x2400", 1)
    assert (rig.canvas_w, rig.canvas_h, rig.n) == (9000, 2400, 8)
    st0 = make_stitcher(1, masks_for_rig(rig), 0)
    assert np.array_equal(gpu_stitch(st0, frames), oracle_lib.Stitch.from_rig(rig, 0).run(frames))


def test_three_images_6000x1800_l6(oracle_lib):
    rig, frames = _full_scale(oracle_lib, "pano3_2704x1520_to_6000x1800", 3)
    assert (rig.canvas_w, rig.canvas_h, rig.n) == (6000, 1800, 3)
    st0 = make_stitcher(3, masks_for_rig(rig), 0)
    assert np.array_equal(gpu_stitch(st0, frames), oracle_lib.Stitch.from_rig(rig, 0).run(frames))


def test_two_images_8500x3300_binomial5_l6(oracle_lib):
    rig, _ = _full_scale(oracle_lib, "pano2_5120x2880_to_8500x3300", 2, filt="binomial5")
    assert (rig.canvas_w, rig.canvas_h) == (8500, 3300)
