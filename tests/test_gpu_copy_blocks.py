"""Copy blocks on the GPU (hmp_stitcher_set_copy_blocks), through the C ABI, against the oracle.

Three- and N-image stitchers copy the write-rect blocks whose reconstruction is exactly one
image's pixel and run the pyramid over the rest. Checked here, bit for bit against the FP32
oracle:
  * copy blocks on after a frame with them off (the level buffers then hold another frame's
    pyramid everywhere, so any read outside the work lists would show);
  * source pixels with alpha 0 (some of them all zero) behind copy blocks, both where the gather
    reads them and where only pyr_down does: the gated fallback recomputes the write rect;
  * frames smaller than the tables' coordinates (the copy blocks' entries leave the frames, so
    the call runs the full pyramid);
  * a CUDA graph of process() replayed on new frames, with and without alpha-0 pixels.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_stitch, lsb_stats, make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu

CASES = [
    # (workload, kind, levels, scale, batch, minimize)
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.5, 1, True),
    ("pano3_2704x1520_to_6000x1800", 3, 6, 0.5, 1, True),
    ("pano3_2704x1520_to_6000x1800", 3, 4, 0.25, 2, True),
    ("panon8_2000x1500_to_9000x2400", 1, 6, 0.5, 1, True),
    ("panon8_2000x1500_to_9000x2400", 1, 5, 0.25, 2, False),
    ("panon8_2000x1500_to_9000x2400", 1, 7, 0.5, 1, True),
    ("pano2_1280x720_to_2200x800", 2, 5, 1.0, 2, True),
]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _exact(out, ref, what):
    if not np.array_equal(out, ref):
        mx, mean = lsb_stats(out, ref)
        bad = np.argwhere(np.abs(out.astype(int) - ref.astype(int)).max(-1) > 0)
        pytest.fail(f"{what}: max {mx} LSB, mean {mean:.6f}, {len(bad)} pixels, first {bad[:5].tolist()}")


@pytest.mark.parametrize("workload,kind,levels,scale,batch,minimize", CASES)
def test_copy_blocks_after_a_full_frame(oracle_lib, workload, kind, levels, scale, batch, minimize):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=31, kind=kind, scale=scale)
    st = make_stitcher(kind, masks_for_rig(rig), levels, batch, minimize)
    assert st.status.ok(), st.status
    info = st.info()
    assert info["copy_mode"] and info["copy_blocks"] > 0 and info["pyramid_blocks"] > 0, info
    o = oracle_lib.Stitch.from_rig(rig, levels, batch, minimize)
    fa = synth.rig_frames(rig, seed=1, batch=batch)
    fb = synth.rig_frames(rig, seed=2, batch=batch)
    st.set_copy_blocks(False)
    _exact(gpu_stitch(st, fa), o.run(fa), "copy blocks off")
    st.set_copy_blocks(True)
    _exact(gpu_stitch(st, fb), o.run(fb), "copy blocks on, after a full frame")
    _exact(gpu_stitch(st, fa), o.run(fa), "copy blocks on, second frame")


def _copied_image(rig, kind, x, y):
    """The image a copy block at canvas (x, y) copies: the label's; with two images image 2 where
    the seam value is 0 and image 2's table covers the pixel, else image 1."""
    label = int(rig.seam[y, x])
    if kind != 2:
        return label
    h, w = rig.map_x[1].shape
    covered = 0 <= x - rig.pos_x[1] < w and 0 <= y - rig.pos_y[1] < h
    return 1 if label == 0 and covered else 0


def _copy_and_pyramid_neighbours(st, rig, kind, levels):
    """Canvas pixels 5 columns right of a copy block's right edge that lie in a pyramid block
    (inside the copy block's reconstruction support), with the image of the copy block."""
    import hmpano

    plan = hmpano.plan_copy_blocks(kind, masks_for_rig(rig), levels)
    cls, (ox, oy) = plan["classes"], plan["origin"]
    pts = []
    for j, i in zip(*np.nonzero(cls[:, :-1] == 0)):
        if cls[j, i + 1] != 1:
            continue
        x, y = ox + 64 * i + 64 + 5, oy + 16 * j + 3
        if x < rig.canvas_w and y < rig.canvas_h:
            pts.append((x, y, _copied_image(rig, kind, x, y)))
    return pts


def _zero_alpha_at(rig, frames, k, x, y, rgb_zero=False):
    """Alpha 0 at the source pixel image k's table maps canvas (x, y) to, if it maps one."""
    rx, ry = x - rig.pos_x[k], y - rig.pos_y[k]
    if not (0 <= ry < rig.map_x[k].shape[0] and 0 <= rx < rig.map_x[k].shape[1]):
        return False
    sx, sy = int(rig.map_x[k][ry, rx]), int(rig.map_y[k][ry, rx])
    if sx >= rig.src_w[k] or sy >= rig.src_h[k]:
        return False
    frames[k][:, sy, sx, 3] = 0
    if rgb_zero:
        frames[k][:, sy, sx, :3] = 0
    return True


@pytest.mark.parametrize("workload,kind,levels,scale,batch,minimize", CASES[:4])
def test_alpha_zero_runs_the_fallback(oracle_lib, workload, kind, levels, scale, batch, minimize):
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=37, kind=kind, scale=scale)
    st = make_stitcher(kind, masks_for_rig(rig), levels, batch, minimize)
    o = oracle_lib.Stitch.from_rig(rig, levels, batch, minimize)
    rng = np.random.default_rng(5)
    # (a) scattered alpha-0 pixels, some of them (0, 0, 0, 0), in every image
    fr = synth.rig_frames(rig, seed=3, batch=batch)
    for k in range(rig.n):
        ys = rng.integers(0, rig.src_h[k], 12)
        xs = rng.integers(0, rig.src_w[k], 12)
        fr[k][:, ys, xs, 3] = 0
        fr[k][:, ys[:4], xs[:4], :3] = 0
    _exact(gpu_stitch(st, fr), o.run(fr), "scattered alpha 0")
    # (b) alpha 0 only behind pyramid-block pixels inside copy blocks' supports (pyr_down's check)
    fr = synth.rig_frames(rig, seed=4, batch=batch)
    pts = _copy_and_pyramid_neighbours(st, rig, kind, levels)
    assert pts, "no copy block next to a pyramid block"
    hit = sum(_zero_alpha_at(rig, fr, k, x, y, rgb_zero=bool(t % 2)) for t, (x, y, k) in enumerate(pts[:6]))
    assert hit > 0
    _exact(gpu_stitch(st, fr), o.run(fr), "alpha 0 behind pyramid blocks")
    # (c) and back to clean frames: the flag is cleared per call
    fr = synth.rig_frames(rig, seed=5, batch=batch)
    _exact(gpu_stitch(st, fr), o.run(fr), "clean frame after a fallback")


@pytest.mark.parametrize("workload,kind,levels,scale,storage,tile_down", [
    ("pano3_2704x1520_to_6000x1800", 3, 6, 0.25, "f16", 64),
    ("panon8_2000x1500_to_9000x2400", 1, 6, 0.25, "f16", 64),
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.5, "f32", 32),
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.5, "f16", 32),
])
def test_alpha_zero_fallback_storage_and_tiles(oracle_lib, workload, kind, levels, scale, storage, tile_down):
    """The fallback's dense chain in the other instantiations it launches: FP16 level storage
    (against the FP64 oracle within the FP16 tolerance) and 32-pixel down tiles."""
    from hmpano import synth

    rig = synth.workload_rig(workload, seed=47, kind=kind, scale=scale)
    st = make_stitcher(kind, masks_for_rig(rig), levels, storage=storage)
    st.set_tiles(tile_down)
    o = oracle_lib.Stitch.from_rig(rig, levels)
    rng = np.random.default_rng(9)
    fr = synth.rig_frames(rig, seed=6)
    for k in range(rig.n):
        ys = rng.integers(0, rig.src_h[k], 16)
        xs = rng.integers(0, rig.src_w[k], 16)
        fr[k][:, ys, xs, 3] = 0
    for what, frames in (("alpha 0", fr), ("clean frame after a fallback", synth.rig_frames(rig, seed=7))):
        out = gpu_stitch(st, frames)
        if storage == "f32":
            _exact(out, o.run(frames), what)
        else:
            mx, mean = lsb_stats(out, o.run(frames, "f64"))
            assert mx <= 1 and mean <= 0.05, (what, mx, mean)


def test_frames_smaller_than_the_tables(oracle_lib):
    """Frames cropped below the tables' coordinates: entries past the frames read as fills, so the
    copy blocks do not apply and the call runs the full pyramid."""
    from hmpano import synth

    rig = synth.workload_rig("panon8_2000x1500_to_9000x2400", seed=41, scale=0.25)
    st = make_stitcher(1, masks_for_rig(rig), 5)
    frames = [np.ascontiguousarray(f[:, : f.shape[1] - 9, : f.shape[2] - 13]) for f in synth.rig_frames(rig, seed=6)]
    _exact(gpu_stitch(st, frames), oracle_lib.Stitch.from_rig(rig, 5).run(frames), "cropped frames")
    full = synth.rig_frames(rig, seed=7)
    _exact(gpu_stitch(st, full), oracle_lib.Stitch.from_rig(rig, 5).run(full), "full frames again")


def test_graph_replay_with_copy_blocks(oracle_lib):
    import torch
    from hmpano import synth

    rig = synth.workload_rig("pano3_2704x1520_to_6000x1800", seed=43, kind=3, scale=0.25)
    st = make_stitcher(3, masks_for_rig(rig), 6)
    o = oracle_lib.Stitch.from_rig(rig, 6)
    f0 = synth.rig_frames(rig, seed=8)
    ins = [torch.from_numpy(f).cuda() for f in f0]
    canvas = torch.zeros((1, rig.canvas_h, rig.canvas_w, 4), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        st._run(ins, canvas, stream=s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st._run(ins, canvas, stream=s)
    for seed, holes in ((9, False), (10, True), (11, False)):
        fr = synth.rig_frames(rig, seed=seed)
        if holes:
            for k in range(rig.n):
                fr[k][:, 100:140, 200:260, 3] = 0
        for t, f in zip(ins, fr):
            t.copy_(torch.from_numpy(f))
        canvas.zero_()
        g.replay()
        torch.cuda.synchronize()
        _exact(canvas.cpu().numpy(), o.run(fr), f"graph replay, seed {seed}")


@pytest.mark.parametrize("workload,kind,levels,scale", [
    ("pano2_5120x2880_to_8500x3300", 2, 6, 0.5),
    ("pano3_2704x1520_to_6000x1800", 3, 6, 0.25),
    ("panon8_2000x1500_to_9000x2400", 1, 6, 0.25),
])
def test_opaque_frames_mode(oracle_lib, workload, kind, levels, scale):
    """Copy blocks for frames promised opaque (mode 2): no alpha check and no fallback launch, and
    on opaque frames the same bits as the oracle; modes switch per call."""
    from hmpano import _lib, synth

    rig = synth.workload_rig(workload, seed=53, kind=kind, scale=scale)
    st = make_stitcher(kind, masks_for_rig(rig), levels)
    o = oracle_lib.Stitch.from_rig(rig, levels)
    checked = st.info()["launches_per_process"]
    st.set_copy_blocks(True, opaque_frames=True)
    assert st.info()["launches_per_process"] == checked - 1
    for seed in (12, 13):
        fr = synth.rig_frames(rig, seed=seed)
        _exact(gpu_stitch(st, fr), o.run(fr), f"opaque frames, seed {seed}")
    st.set_copy_blocks(True)
    fr = synth.rig_frames(rig, seed=14)
    _exact(gpu_stitch(st, fr), o.run(fr), "checked mode after opaque mode")
    for bad in (-1, 3):
        s = _lib.lib().hmp_stitcher_set_copy_blocks(st._handle, bad)
        assert s.code == 1, bad
