"""The batched streaming form (hmpano/batch.py): the whole multi-stream job replayed from one
CUDA graph, at several frames-per-call and tile choices, gives every stream's frames exactly as
the plain per-frame path does (same kernels per frame: bit for bit)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_batched_graph_job_equals_plain_path():
    import build as hmp_build
    import torch

    from hmpano import batch

    hmp_build.build()
    dev = torch.device("cuda", 0)
    job = batch.Job(dev, frames=4, scale=0.25)
    _, want = batch.plain_path(job, keep_last=True)
    for b, tile in [(1, 32), (2, 64), (4, 32)]:
        plan = batch.Plan(job, b, tile)
        plan.time(1)
        got = plan.last_canvases()
        for i, (g, w) in enumerate(zip(got, want)):
            assert torch.equal(g, w), (b, tile, i)
    tune = batch.autotune(job, batches=(1, 2), tiles=(32, 64), reps=1, use_cache=False)
    assert tune["batch"] in (1, 2) and tune["tile_down"] in (32, 64) and len(tune["trials"]) == 4
