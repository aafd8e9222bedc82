"""GPU parity: the sm_103a stitching kernels, called through the C ABI, against the oracle.

FP32 storage reproduces the reference's operation order (no fused multiply-add, IEEE division),
so every FP32 result must equal the FP32 oracle bit for bit; the oracle itself equals the
reference's golden vectors bit for bit (test_oracle_golden.py). FP16 pyramid storage is
checked against the FP64 oracle with a tolerance of 1 uint8 LSB (max) and 0.05 LSB (mean).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_stitch, lsb_stats, make_stitcher, masks_for_case, masks_for_rig

pytestmark = pytest.mark.gpu

F16_MAX_LSB = 1
F16_MEAN_LSB = 0.05


@pytest.fixture(scope="module", autouse=True)
def _built():
    import sys
    from pathlib import Path

    import torch

    repo = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(repo / "hm-cupano_gb300"))
    import build as hmp_build

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _golden_names(golden):
    return [str(n) for n in golden["names"]]


def test_golden_cases_bit_exact(golden, oracle_lib):
    for name in _golden_names(golden):
        c = oracle_lib.load_golden_case(golden, name)
        st = make_stitcher(c["kind"], masks_for_case(c), c["levels"], c["batch"], c["minimize"])
        assert st.status.ok(), (name, st.status)
        out = gpu_stitch(st, c["frames"])
        assert out.shape == c["canvas"].shape, name
        if not np.array_equal(out, c["canvas"]):
            mx, mean = lsb_stats(out, c["canvas"])
            pytest.fail(f"{name}: differs from the reference (max {mx} LSB, mean {mean:.4f})")


def test_golden_cases_f16_storage(golden, oracle_lib):
    for name in _golden_names(golden):
        c = oracle_lib.load_golden_case(golden, name)
        if c["levels"] < 2 or c["frames"][0].shape[-1] != 4:  # FP16 storage is an RGBA8 option
            continue
        st = make_stitcher(c["kind"], masks_for_case(c), c["levels"], c["batch"], c["minimize"], storage="f16")
        out = gpu_stitch(st, c["frames"])
        ref = oracle_lib.Stitch(c["kind"], c["map_x"], c["map_y"], c["pos_x"], c["pos_y"], c["seam"], c["levels"],
                                c["batch"], c["minimize"]).run(c["frames"], "f64")
        mx, mean = lsb_stats(out, ref)
        assert mx <= F16_MAX_LSB and mean <= F16_MEAN_LSB, (name, mx, mean)


WORKLOADS = [
    # (workload, kind, levels, scale, minimize, batch, extra rig kwargs)
    ("pano2_1280x720_to_2200x800", 2, 0, 1.0, True, 1, {}),
    ("pano2_1280x720_to_2200x800", 2, 6, 1.0, True, 1, {}),
    ("pano2_1280x720_to_2200x800", 2, 4, 1.0, False, 1, {}),
    ("pano2_1280x720_to_2200x800", 2, 5, 1.0, True, 2, {"oob_fraction": 0.02}),
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.25, True, 1, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 0, 0.25, True, 1, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 6, 0.25, True, 1, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 6, 0.25, False, 1, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 3, 0.25, True, 2, {"oob_fraction": 0.02}),
    ("pano3_2704x1520_to_6000x1800", 3, 0, 0.25, True, 1, {}),
    ("pano3_2704x1520_to_6000x1800", 3, 6, 0.25, True, 1, {}),
    ("pano3_2704x1520_to_6000x1800", 1, 6, 0.25, True, 1, {}),
    ("pano3_2704x1520_to_6000x1800", 3, 4, 0.25, True, 1, {"oob_fraction": 0.02}),
    ("pano3_2704x1520_to_6000x1800", 3, 2, 0.25, True, 2, {}),
    ("panon8_2000x1500_to_9000x2400", 1, 2, 0.25, True, 1, {}),
]


@pytest.mark.parametrize("workload,kind,levels,scale,minimize,batch,rkw", WORKLOADS)
def test_workloads_match_oracle(oracle_lib, workload, kind, levels, scale, minimize, batch, rkw):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=17, kind=kind, scale=scale, **rkw)
    frames = synth.rig_frames(rig, seed=5, batch=batch)
    st = make_stitcher(kind, masks_for_rig(rig), levels, batch, minimize)
    assert st.status.ok(), st.status
    out = gpu_stitch(st, frames)
    ref = oracle_lib.Stitch.from_rig(rig, levels, batch, minimize).run(frames)
    if not np.array_equal(out, ref):
        mx, mean = lsb_stats(out, ref)
        bad = np.argwhere(np.abs(out.astype(int) - ref.astype(int)).max(-1) > 0)
        pytest.fail(f"differs from the oracle: max {mx} LSB, mean {mean:.5f}, first pixels {bad[:5].tolist()}")


def test_three_image_legacy_remap(oracle_lib):
    # fused=False keeps the opaque (alpha 255) rule for out-of-range table entries.
    import hmpano
    from hmpano import synth

    rig = synth.workload_rig("pano3_2704x1520_to_6000x1800", seed=3, kind=3, scale=0.25, oob_fraction=0.05)
    frames = synth.rig_frames(rig, seed=9)
    for fused in (True, False):
        st = hmpano.CudaStitchPano3(1, 4, masks_for_rig(rig), quiet=True, fused=fused)
        out = gpu_stitch(st, frames)
        ref = oracle_lib.Stitch.from_rig(rig, 4, fused3=fused).run(frames)
        assert np.array_equal(out, ref), fused
    # The reference picks the mode per call: process(..., fused) (src/pano/cudaPano3.h:101-107).
    import torch

    st = hmpano.CudaStitchPano3(1, 4, masks_for_rig(rig), quiet=True)
    ins = [torch.from_numpy(f).cuda() for f in frames]
    for fused in (False, True, False):
        out = st.process(*ins, fused=fused).cpu().numpy()
        assert np.array_equal(out, oracle_lib.Stitch.from_rig(rig, 4, fused3=fused).run(frames)), fused


def test_full_scale_two_image_l6():
    """Two 5120x2880 frames onto 8500x3300 with 6 levels (the production configuration)."""
    from oracle import oracle as O
    from hmpano import synth

    rig = synth.workload_rig("pano2_5120x2880_to_8500x3300", seed=1234)
    frames = synth.rig_frames(rig, seed=1)
    assert (rig.canvas_w, rig.canvas_h) == (8500, 3300)
    o = O.Stitch.from_rig(rig, 6)
    st = make_stitcher(2, masks_for_rig(rig), 6)
    out = gpu_stitch(st, frames)
    ref = o.run(frames)
    mx, mean = lsb_stats(out, ref)
    assert mx == 0, (mx, mean)
    st16 = make_stitcher(2, masks_for_rig(rig), 6, storage="f16")
    out16 = gpu_stitch(st16, frames)
    ref64 = o.run(frames, "f64")
    mx, mean = lsb_stats(out16, ref64)
    assert mx <= F16_MAX_LSB and mean <= F16_MEAN_LSB, (mx, mean)
    # the hard seam of the same rig
    st0 = make_stitcher(2, masks_for_rig(rig), 0)
    assert np.array_equal(gpu_stitch(st0, frames), O.Stitch.from_rig(rig, 0).run(frames))


def test_pitched_and_unaligned_buffers(oracle_lib):
    """Row pitch larger than 4*width for inputs and canvas, and a canvas that is not 16-byte
    aligned (the kernels fall back from 128-bit stores)."""
    import torch
    from hmpano import synth

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=8)
    frames = synth.rig_frames(rig, seed=2, batch=2)
    ref = oracle_lib.Stitch.from_rig(rig, 5, 2).run(frames)
    st = make_stitcher(2, masks_for_rig(rig), 5, 2)
    ins = []
    for f in frames:
        B, H, W, _ = f.shape
        big = torch.zeros((B, H, W + 7, 4), dtype=torch.uint8, device="cuda")
        big[:, :, :W] = torch.from_numpy(f).cuda()
        ins.append(big[:, :, :W])
    W, H = rig.canvas_w, rig.canvas_h
    store = torch.zeros((2 * H * (W + 3) * 4 + 4,), dtype=torch.uint8, device="cuda")
    canvas = store[4:4 + 2 * H * (W + 3) * 4].view(2, H, W + 3, 4)[:, :, :W]
    out = st._run(ins, canvas)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


def test_deterministic_and_no_state_leak(oracle_lib):
    from hmpano import synth

    rig = synth.workload_rig("panon8_2000x1500_to_9000x2400", seed=4, scale=0.25)
    st = make_stitcher(1, masks_for_rig(rig), 5)
    f1 = synth.rig_frames(rig, seed=1)
    f2 = synth.rig_frames(rig, seed=2)
    a = gpu_stitch(st, f1)
    b = gpu_stitch(st, f2)
    c = gpu_stitch(st, f1)
    assert np.array_equal(a, c)
    assert np.array_equal(b, oracle_lib.Stitch.from_rig(rig, 5).run(f2))


def test_process_errors_are_sticky():
    import torch
    import hmpano
    from hmpano import synth

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=8)
    st = make_stitcher(2, masks_for_rig(rig), 3)
    frames = [torch.from_numpy(f).cuda() for f in synth.rig_frames(rig, seed=2)]
    bad_canvas = torch.zeros((1, 10, 10, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(hmpano.CudaStatusError):
        st.process(frames[0], frames[1], bad_canvas)
    assert not st.status.ok()
    with pytest.raises(hmpano.CudaStatusError):  # sticky, like CudaStatus::Update
        st.process(frames[0], frames[1])


def test_reference_backend_names(oracle_lib):
    """The reference's backend names run these kernels (same bits); an unknown one is its
    ValueError from process() (cupano/ops.py:60-69)."""
    import torch
    from hmpano import synth

    import hmpano

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=8)
    frames = [torch.from_numpy(f).cuda() for f in synth.rig_frames(rig, seed=2)]
    outs = []
    for backend in ("auto", "triton"):
        st = hmpano.CudaStitchPano(1, 3, masks_for_rig(rig), True, True, 0, backend, False)
        outs.append(st.process(frames[0], frames[1]).cpu())
    assert torch.equal(outs[0], outs[1])
    st = hmpano.CudaStitchPano(1, 3, masks_for_rig(rig), quiet=True, backend="torch")
    with pytest.raises(ValueError, match="Unsupported backend"):
        st.process(frames[0], frames[1])


def test_graph_capture_replays_identically(oracle_lib):
    """process() allocates nothing, so it can be captured in a CUDA graph and replayed."""
    import torch
    from hmpano import synth

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=12)
    frames = synth.rig_frames(rig, seed=4)
    st = make_stitcher(2, masks_for_rig(rig), 6)
    ins = [torch.from_numpy(f).cuda() for f in frames]
    canvas = torch.zeros((1, rig.canvas_h, rig.canvas_w, 4), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        st._run(ins, canvas, stream=s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st._run(ins, canvas, stream=s)
    canvas.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(canvas.cpu().numpy(), oracle_lib.Stitch.from_rig(rig, 6).run(frames))
