"""Stitcher-level layouts of the reference's GTests, re-expressed as data: identity remaps, the
tests' pattern frames and seams (src/pano/cudaPanoN_test.cpp:192-298). Each layout is checked
for minimize == full and, where the reference does, for a transparent gap; test_oracle_golden.py
runs them on the oracle, test_gpu_layouts.py on the GPU.
"""
from __future__ import annotations

import numpy as np

KIND_PANON = 1


def identity_maps(w: int, h: int):
    return (np.tile(np.arange(w, dtype=np.uint16), (h, 1)),
            np.tile(np.arange(h, dtype=np.uint16)[:, None], (1, w)))


def pattern_frame(w: int, h: int, idx: int) -> np.ndarray:
    """The tests' pattern: base 50 * idx plus x % 17, y % 19, (x + y) % 23; alpha 255. Every value
    is an integer below 256, so the same frame serves the uint8 and float pipelines."""
    x = np.arange(w)[None, :]
    y = np.arange(h)[:, None]
    f = np.zeros((h, w, 4), np.float32)
    f[..., 0] = 50 * idx + x % 17
    f[..., 1] = 50 * idx + y % 19
    f[..., 2] = 50 * idx + (x + y) % 23
    f[..., 3] = 255
    return f


def layouts():
    """name -> dict(sizes, positions, seam, levels, gap) for the four N-image layouts."""
    out = {}
    # Two images on the same footprint, seam down the middle (:192-212).
    W = H = 384
    seam = np.zeros((H, W), np.uint8)
    seam[:, W // 2:] = 1
    out["two_way_overlap"] = dict(sizes=[(W, H)] * 2, positions=[(0, 0), (0, 0)], seam=seam, levels=4, gap=None)
    # Two images butted with no overlap (:214-234).
    W, H = 192, 384
    seam = np.zeros((H, 2 * W), np.uint8)
    seam[:, W:] = 1
    out["no_overlap"] = dict(sizes=[(W, H)] * 2, positions=[(0, 0), (W, 0)], seam=seam, levels=4, gap=None)
    # Two images with an uncovered gap [128, 256) between them, which stays transparent (:236-261).
    W, H, CW = 128, 384, 384
    seam = np.zeros((H, CW), np.uint8)
    seam[:, CW // 2:] = 1
    out["gap"] = dict(sizes=[(W, H)] * 2, positions=[(0, 0), (2 * W, 0)], seam=seam, levels=4, gap=(W, 2 * W))
    # Four images on one footprint; label 0 except a central 64x64 square split into quadrants
    # 0..3, so that four seams meet at its centre (:263-298).
    W = H = 384
    seam = np.zeros((H, W), np.uint8)
    cx, cy, half = W // 2, H // 2, 32
    ys, xs = np.mgrid[cy - half:cy + half, cx - half:cx + half]
    seam[cy - half:cy + half, cx - half:cx + half] = ((ys >= cy).astype(np.uint8) * 2 + (xs >= cx)).astype(np.uint8)
    out["multi_seam_intersection"] = dict(sizes=[(W, H)] * 4, positions=[(0, 0)] * 4, seam=seam, levels=4, gap=None)
    return out


def tables(layout):
    mx, my = zip(*[identity_maps(w, h) for w, h in layout["sizes"]])
    return list(mx), list(my)


def frames(layout, dtype=np.uint8):
    return [pattern_frame(w, h, i).astype(dtype)[None] for i, (w, h) in enumerate(layout["sizes"])]
