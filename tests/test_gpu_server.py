"""The continuous-batching stitch server (hmp_server_*): each result in a mix of configurations,
submitted in shuffled order and overlapping on the GPU, equals the same request stitched alone
(bit for bit: both run the same kernels on the same inputs); a tight HBM budget forces
evictions and is never exceeded; waits are bounded and errors come back as statuses."""
from __future__ import annotations

import random

import numpy as np
import pytest

from helpers import make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu

CONFIGS = [
    # (workload, kind, levels, scale)
    ("pano2_1280x720_to_2200x800", 2, 6, 1.0),
    ("pano3_2704x1520_to_6000x1800", 3, 4, 0.25),
    ("panon8_2000x1500_to_9000x2400", 1, 3, 0.25),
    ("pano2_1280x720_to_2200x800", 2, 0, 1.0),
]


@pytest.fixture(scope="module")
def prepared():
    import build as hmp_build
    import torch

    from hmpano import synth
    from oracle import oracle

    hmp_build.build()
    oracle.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    out = []
    for ci, (workload, kind, levels, scale) in enumerate(CONFIGS):
        rig = synth.workload_rig(workload, seed=100 + ci, kind=kind, scale=scale)
        alone = make_stitcher(kind, masks_for_rig(rig), levels)
        assert alone.status.ok(), alone.status
        sets = []
        for s in range(3):
            host = synth.rig_frames(rig, seed=1000 * ci + s)
            frames = [torch.from_numpy(f).cuda() for f in host]
            ref = alone._run(frames).clone()
            if s == 0:  # the request alone is itself the oracle's result, bit for bit (FP32 storage)
                want = oracle.Stitch.from_rig(rig, levels).run(host)
                assert np.array_equal(ref.cpu().numpy(), want), workload
            sets.append((frames, ref))
        torch.cuda.synchronize()
        out.append({"rig": rig, "kind": kind, "levels": levels, "sets": sets,
                    "canvas": (alone.canvas_height(), alone.canvas_width()), "bytes": alone.info()["device_bytes"]})
    return out


def _server(prepared, budget, slots=3, per_config=2):
    import hmpano

    srv = hmpano.StitchServer(budget, slots=slots, max_instances_per_config=per_config)
    ids = [srv.add_config(p["kind"], masks_for_rig(p["rig"]), p["levels"]) for p in prepared]
    return srv, ids


def _run_mix(srv, ids, prepared, order):
    import torch

    outs = []
    for ci, si in order:
        h, w = prepared[ci]["canvas"]
        canvas = torch.full((1, h, w, 4), 7, dtype=torch.uint8, device="cuda")
        rid = srv.submit(ids[ci], prepared[ci]["sets"][si][0], canvas)
        outs.append((rid, ci, si, canvas))
    st = srv.drain(120000)
    assert st.ok(), st
    for rid, ci, si, canvas in outs:
        assert torch.equal(canvas, prepared[ci]["sets"][si][1]), (ci, si)


def test_server_mix_equals_alone(prepared):
    srv, ids = _server(prepared, budget=64 << 30)
    order = [(ci, si) for ci in range(len(CONFIGS)) for si in range(3)] * 2
    random.Random(7).shuffle(order)
    _run_mix(srv, ids, prepared, order)
    s = srv.stats()
    assert s["completed"] == len(order) and s["failed"] == 0
    assert s["max_in_flight"] >= 2  # requests overlapped on the GPU
    assert 0 < s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["instances_evicted"] == 0
    srv.close()


def test_server_evicts_within_budget(prepared):
    sizes = sorted(p["bytes"] for p in prepared)
    budget = int(sizes[-1] + sizes[-2] * 0.5)  # the two largest never fit together
    srv, ids = _server(prepared, budget=budget, slots=2, per_config=1)
    order = [(ci % len(CONFIGS), ci % 3) for ci in range(16)]
    _run_mix(srv, ids, prepared, order)
    s = srv.stats()
    assert s["completed"] == len(order) and s["failed"] == 0
    assert s["instances_evicted"] > 0
    assert s["resident_bytes_peak"] <= budget
    srv.close()


def test_server_bounded_waits_and_errors(prepared):
    import torch

    from hmpano import CudaStatusError

    srv, ids = _server(prepared, budget=int(min(p["bytes"] for p in prepared) // 2))
    st = srv.wait(123456, timeout_ms=50)  # unknown request: bounded wait
    assert st.code == 909
    p = prepared[0]
    with pytest.raises(CudaStatusError):
        srv.submit(ids[0], p["sets"][0][0][:1], torch.empty((1, *p["canvas"], 4), dtype=torch.uint8, device="cuda"))
    h, w = p["canvas"]
    rid = srv.submit(ids[0], p["sets"][0][0], torch.empty((1, h, w, 4), dtype=torch.uint8, device="cuda"))
    st = srv.wait(rid, timeout_ms=60000)  # larger than the whole budget: fails, does not hang
    assert st.code == 2, st
    # Its size is now known: a second request of the configuration fails at once as well.
    rid = srv.submit(ids[0], p["sets"][0][0], torch.empty((1, h, w, 4), dtype=torch.uint8, device="cuda"))
    st = srv.wait(rid, timeout_ms=60000)
    assert st.code == 2, st
    assert srv.drain(10000).ok()
    srv.close()
