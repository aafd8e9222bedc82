"""The batched streaming form (hmpano/batch.py): the whole multi-stream job replayed from one
CUDA graph, at several frames-per-call and tile choices, gives every stream's frames exactly as
the plain per-frame path does (same kernels per frame: bit for bit)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def _check_against_oracle(job, canvases):
    """One stream of each kind (two- and three-image): its last frame's canvas against the FP64
    oracle on the same frames, within the FP16-storage tolerance (1 LSB max, 0.05 LSB mean)."""
    import numpy as np
    from oracle import oracle

    oracle.build()
    seen = set()
    for s, c in zip(job.streams, canvases):
        if s["kind"] in seen:
            continue
        seen.add(s["kind"])
        frames = [t[job.frames - 1:job.frames].cpu().numpy() for t in s["inputs"]]
        ref = oracle.Stitch.from_rig(s["rig"], job.levels).run(frames, "f64")[0]
        d = np.abs(c.cpu().numpy().astype(np.int32) - ref.astype(np.int32))
        assert int(d.max()) <= 1 and float(d.mean()) <= 0.05, (s["workload"], int(d.max()), float(d.mean()))
    assert seen == {2, 3}


def test_batched_graph_job_equals_plain_path():
    import build as hmp_build
    import torch

    from hmpano import batch

    hmp_build.build()
    dev = torch.device("cuda", 0)
    job = batch.Job(dev, frames=4, scale=0.25)
    _, want = batch.plain_path(job, keep_last=True)
    _check_against_oracle(job, want)
    for b, tile in [(1, 32), (2, 64), (4, 32)]:
        plan = batch.Plan(job, b, tile)
        plan.time(1)
        got = plan.last_canvases()
        for i, (g, w) in enumerate(zip(got, want)):
            assert torch.equal(g, w), (b, tile, i)
    tune = batch.autotune(job, batches=(1, 2), tiles=(32, 64), reps=1, use_cache=False)
    # 2 batches x (two-image: 32, 64, 64 capped at 4 CTAs per SM) x (three-image: the same)
    assert tune["batch"] in (1, 2) and len(tune["trials"]) == 18
    assert set(tune["tile_down"]) == {"2", "3"}
    assert all(v[0] in (32, 64) and v[1] in (0, 4) for v in tune["tile_down"].values())
    plan = batch.Plan(job, 2, {2: 64, 3: 32})
    plan.time(1)
    for i, (g, w) in enumerate(zip(plan.last_canvases(), want)):
        assert torch.equal(g, w), ("per-kind tiles", i)


def test_native_batch_replays_with_refilled_inputs():
    """hmp_batch_*: the captured job reads its inputs at launch, so refilled inputs give new canvases
    equal to process() on them; calls on two stream indices both run."""
    import torch

    import hmpano
    from hmpano import synth

    from helpers import make_stitcher, masks_for_rig

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=12, kind=2, scale=0.5)
    st = make_stitcher(2, masks_for_rig(rig), 4, 1)
    st2 = make_stitcher(2, masks_for_rig(rig), 4, 1)  # one process() in flight per stitcher
    frames = [torch.from_numpy(f).cuda() for f in synth.rig_frames(rig, seed=2)]
    other = [torch.from_numpy(f).cuda() for f in synth.rig_frames(rig, seed=3)]
    h, w = st.canvas_height(), st.canvas_width()
    cv = [torch.empty((1, h, w, 4), dtype=torch.uint8, device="cuda") for _ in range(2)]
    job = hmpano.Batch()
    job.add(st, frames, cv[0], stream_index=0)
    job.add(st2, other, cv[1], stream_index=1)
    with pytest.raises(hmpano.CudaStatusError, match="stream index"):
        job.add(st, other, cv[1], stream_index=1)
    job.launch()
    torch.cuda.synchronize()
    assert torch.equal(cv[0], st.process(*frames)) and torch.equal(cv[1], st.process(*other))
    for f in frames:
        f.copy_(torch.roll(f, shifts=5, dims=2))
    job.launch()
    torch.cuda.synchronize()
    assert torch.equal(cv[0], st.process(*frames))
    job.close()
