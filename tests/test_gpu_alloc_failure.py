"""Construction failures, injected on the host: every device allocation a stitcher makes at
construction is failed in turn (hmp_debug_fail_allocation), and each time

  * the constructor keeps cudaErrorMemoryAllocation (2) as the stitcher's sticky status, naming
    what it was allocating, and releases everything it had allocated;
  * process() returns that status without touching the canvas (nothing is launched), and keeps
    returning it (src/pano/cudaPano.inl:28-31, 460-472);
  * a stitcher made after the injection is switched off works and matches the oracle.

No device call fails for real: the failure is a status the library's allocator returns.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_stitch, make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


@pytest.mark.parametrize("workload,kind,levels", [
    ("pano3_2704x1520_to_6000x1800", 3, 4),
    ("pano2_1280x720_to_2200x800", 2, 5),
    ("panon8_2000x1500_to_9000x2400", 1, 3),
])
def test_every_construction_allocation_failure_is_sticky(oracle_lib, workload, kind, levels):
    import torch

    import hmpano
    from hmpano import _lib, synth

    lib = _lib.lib()
    rig = synth.workload_rig(workload, seed=21, kind=kind, scale=0.25 if kind != 2 else 0.5)
    masks = masks_for_rig(rig)
    frames = synth.rig_frames(rig, seed=2)
    ins = [torch.from_numpy(f).cuda() for f in frames]
    c0 = lib.hmp_debug_allocation_count()
    good = make_stitcher(kind, masks, levels)
    assert good.status.ok(), good.status
    n = lib.hmp_debug_allocation_count() - c0
    assert n >= 5, n
    del good
    h, w = rig.canvas_h, rig.canvas_w
    try:
        for k in range(1, n + 1):
            lib.hmp_debug_fail_allocation(k)
            bad = make_stitcher(kind, masks, levels)
            lib.hmp_debug_fail_allocation(0)
            st = bad.status
            assert st.code == 2, (k, st)
            assert bad.info()["device_bytes"] == 0, (k, bad.info()["device_bytes"])
            canvas = torch.full((1, h, w, 4), 77, dtype=torch.uint8, device="cuda")
            for _ in range(2):  # sticky: the same error on every call
                with pytest.raises(hmpano.CudaStatusError) as err:
                    bad._run(ins, canvas)
                assert err.value.status.code == 2, (k, err.value.status)
            torch.cuda.synchronize()
            assert bool((canvas == 77).all()), k  # nothing ran
    finally:
        lib.hmp_debug_fail_allocation(0)
    after = make_stitcher(kind, masks, levels)
    assert after.status.ok(), after.status
    assert np.array_equal(gpu_stitch(after, frames), oracle_lib.Stitch.from_rig(rig, levels).run(frames))
