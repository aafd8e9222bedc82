"""Copy blocks, checked on the CPU against the oracle (no GPU): the blocks the planner classifies as
copy must equal, in the oracle's full FP32 pyramid blend, the label image's pixel (the hard seam's
result), and the empty ones (0, 0, 0, 0), on random three- and N-image rigs of every supported
depth. This pins the exactness argument the stitchers rely on when they copy those blocks instead
of running the pyramid there (hm-cupano_gb300/csrc/hmp_copyplan.h)."""
from __future__ import annotations

import numpy as np

from helpers import masks_for_rig


def test_copy_blocks_equal_the_oracle_pyramid(oracle_lib):
    import hmpano
    from hmpano import synth

    rng = np.random.default_rng(20261204)
    copies = empties = rigs = 0
    for trial in range(36):
        n = int(rng.integers(3, 9))
        kind = 3 if n == 3 and trial % 2 == 0 else 1
        cw = int(rng.integers(500, 1400))
        ch = int(rng.integers(200, 520))
        sw = int(rng.integers(cw // n + 40, cw // n + 200))
        sh = int(rng.integers(int(ch * 0.7), ch))
        rig = synth.make_rig(cw, ch, n, sw, sh, float(rng.uniform(0.15, 0.35)), seed=int(rng.integers(1 << 30)),
                             kind=kind)
        levels = int(rng.integers(2, 8))
        minimize = bool(trial % 3 != 0)
        masks = masks_for_rig(rig)
        plan = hmpano.plan_copy_blocks(kind, masks, levels, minimize)
        if plan["classes"] is None:
            continue
        geo = hmpano.plan_geometry(kind, masks, levels, minimize)
        wx, wy, ww, wh = geo["write"]
        frames = synth.rig_frames(rig, seed=trial)
        out = oracle_lib.Stitch.from_rig(rig, levels, 1, minimize).run(frames)[0]
        hard = oracle_lib.Stitch.from_rig(rig, 0).run(frames)[0]
        ox, oy = plan["origin"]
        cls = plan["classes"]
        rigs += 1
        for j, i in zip(*np.nonzero(cls != 1)):
            x0, x1 = max(ox + 64 * i, wx), min(ox + 64 * i + 64, wx + ww)
            y0, y1 = max(oy + 16 * j, wy), min(oy + 16 * j + 16, wy + wh)
            got = out[y0:y1, x0:x1]
            if cls[j, i] == 0:
                copies += 1
                want = hard[y0:y1, x0:x1]
            else:
                empties += 1
                want = np.zeros_like(got)
            assert np.array_equal(got, want), (trial, n, kind, levels, minimize, (i, j), int(cls[j, i]))
    assert rigs >= 20 and copies > 1000 and empties > 0, (rigs, copies, empties)


def _last_writer(rig, frames):
    """Canvas of the two-image rule outside the blend strip: image 2's table where it covers,
    else image 1's (source pixel where the entry lies in the frame, else 0)."""
    out = np.zeros((rig.canvas_h, rig.canvas_w, 4), np.uint8)
    for k in (0, 1):
        mx, my = rig.map_x[k].astype(np.int64), rig.map_y[k].astype(np.int64)
        h, w = mx.shape
        f = frames[k][0]
        ok = (mx < f.shape[1]) & (my < f.shape[0])
        px = np.zeros((h, w, 4), np.uint8)
        px[ok] = f[my[ok], mx[ok]]
        out[rig.pos_y[k]:rig.pos_y[k] + h, rig.pos_x[k]:rig.pos_x[k] + w] = px
    return out


def test_two_image_copy_blocks_equal_the_oracle_pyramid(oracle_lib):
    import hmpano
    from hmpano import synth

    rng = np.random.default_rng(77)
    copies = rigs = 0
    for trial in range(16):
        cw = int(rng.integers(700, 1600))
        ch = int(rng.integers(200, 500))
        sw = int(rng.integers(cw // 2 + 60, cw // 2 + 260))
        sh = int(rng.integers(int(ch * 0.7), ch))
        rig = synth.make_rig(cw, ch, 2, sw, sh, float(rng.integers(200, 320)), seed=int(rng.integers(1 << 30)), kind=2)
        levels = int(rng.integers(2, 8))
        masks = masks_for_rig(rig)
        plan = hmpano.plan_copy_blocks(2, masks, levels, True)
        if plan["classes"] is None:
            continue
        geo = hmpano.plan_geometry(2, masks, levels, True)
        wx, wy, ww, wh = geo["write"]
        frames = synth.rig_frames(rig, seed=trial)
        out = oracle_lib.Stitch.from_rig(rig, levels, 1, True).run(frames)[0]
        lw = _last_writer(rig, frames)
        ox, oy = plan["origin"]
        cls = plan["classes"]
        rigs += 1
        for j, i in zip(*np.nonzero(cls != 1)):
            x0, x1 = max(ox + 64 * i, wx), min(ox + 64 * i + 64, wx + ww)
            y0, y1 = max(oy + 16 * j, wy), min(oy + 16 * j + 16, wy + wh)
            want = lw[y0:y1, x0:x1] if cls[j, i] == 0 else np.zeros_like(out[y0:y1, x0:x1])
            copies += int(cls[j, i] == 0)
            assert np.array_equal(out[y0:y1, x0:x1], want), (trial, levels, (i, j), int(cls[j, i]))
    assert rigs >= 10 and copies > 200, (rigs, copies)


def test_copy_blocks_cover_most_of_the_named_rigs():
    """The three-image stream of the batched workload and the eight-image rig: most write-rect
    blocks are copies, and a good part of the two-image strip. A two-image blend over the whole
    canvas, N-image stitchers of two images and one-level pyramids have none."""
    import hmpano
    from hmpano import synth

    for name, kind, floor in (("pano3_2704x1520_to_6000x1800", 3, 0.7), ("panon8_2000x1500_to_9000x2400", 1, 0.5)):
        rig = synth.workload_rig(name, seed=1234, kind=kind, scale=0.5)
        plan = hmpano.plan_copy_blocks(kind, masks_for_rig(rig), 6)
        cls = plan["classes"]
        assert cls is not None and float((cls == 0).mean()) > floor, (name, float((cls == 0).mean()))
    rig = synth.workload_rig("pano2_5120x2880_to_8500x3300", seed=1234, scale=0.5)
    cls = hmpano.plan_copy_blocks(2, masks_for_rig(rig), 6)["classes"]
    assert cls is not None and float((cls == 0).mean()) > 0.25, float((cls == 0).mean())
    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=3)
    assert hmpano.plan_copy_blocks(2, masks_for_rig(rig), 6, False)["classes"] is None  # no strip
    rig = synth.workload_rig("pano3_2704x1520_to_6000x1800", seed=3, kind=3, scale=0.25)
    assert hmpano.plan_copy_blocks(3, masks_for_rig(rig), 1)["classes"] is None
    rig = synth.make_rig(600, 300, 2, 400, 280, 0.3, seed=5, kind=1)  # N-image stitcher of two images
    assert hmpano.plan_copy_blocks(1, masks_for_rig(rig), 4, False)["classes"] is None
