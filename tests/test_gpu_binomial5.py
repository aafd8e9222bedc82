"""GPU parity of the Binomial5 pyramid (5-tap [1,4,6,4,1]/16, reflect-101; no reference
implementation, so parity is against the oracle alone).

FP32 storage follows the oracle's operation order term by term, so it must equal the FP32 oracle
bit for bit; FP16 storage is checked against the FP64 oracle with the FP16 tolerance of the
parity tests (1 uint8 LSB max, 0.05 LSB mean).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_stitch, lsb_stats, make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu

F16_MAX_LSB = 1
F16_MEAN_LSB = 0.05

CASES = [
    # (workload, kind, levels, scale, minimize, batch)
    ("pano2_1280x720_to_2200x800", 2, 6, 1.0, True, 1),
    ("pano2_1280x720_to_2200x800", 2, 3, 1.0, False, 2),
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.25, True, 1),
    ("pano3_2704x1520_to_6000x1800", 3, 4, 0.25, True, 1),
    ("panon8_2000x1500_to_9000x2400", 1, 5, 0.25, True, 1),
    ("panon8_2000x1500_to_9000x2400", 1, 2, 0.25, False, 1),
    # 7 levels of small rigs: the coarsest levels are a few pixels across, narrower than the
    # filter's staged tiles
    ("pano2_1280x720_to_2200x800", 2, 7, 0.25, True, 1),
    ("panon8_2000x1500_to_9000x2400", 1, 7, 0.125, True, 1),
]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


@pytest.mark.parametrize("workload,kind,levels,scale,minimize,batch", CASES)
def test_binomial5_matches_oracle(oracle_lib, workload, kind, levels, scale, minimize, batch):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=23, kind=kind, scale=scale)
    frames = synth.rig_frames(rig, seed=8, batch=batch)
    st = make_stitcher(kind, masks_for_rig(rig), levels, batch, minimize, filter="binomial5")
    assert st.status.ok(), st.status
    out = gpu_stitch(st, frames)
    ref = oracle_lib.Stitch.from_rig(rig, levels, batch, minimize, filter=oracle_lib.FILTER_BINOMIAL5).run(frames)
    if not np.array_equal(out, ref):
        mx, mean = lsb_stats(out, ref)
        pytest.fail(f"differs from the FP32 oracle: max {mx} LSB, mean {mean:.5f}")


@pytest.mark.parametrize("workload,kind,levels,scale,minimize,batch", CASES[::2])
def test_binomial5_f16_storage_within_one_lsb_of_f64(oracle_lib, workload, kind, levels, scale, minimize, batch):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=29, kind=kind, scale=scale)
    frames = synth.rig_frames(rig, seed=4, batch=batch)
    st = make_stitcher(kind, masks_for_rig(rig), levels, batch, minimize, filter="binomial5", storage="f16")
    assert st.status.ok(), st.status
    out = gpu_stitch(st, frames)
    ref = oracle_lib.Stitch.from_rig(rig, levels, batch, minimize, filter=oracle_lib.FILTER_BINOMIAL5).run(frames, "f64")
    mx, mean = lsb_stats(out, ref)
    assert mx <= F16_MAX_LSB and mean <= F16_MEAN_LSB, (mx, mean)
