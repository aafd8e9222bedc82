"""Stabiliser timings on the GPU: the reference's three steps (Harris corners, Lucas-Kanade flow,
warp; src/cuda/cudaStabilize.cu:274-314) per frame pair, each step timed with CUDA events.

Frames are seeded synthetic grayscale textures moved by a whole-pixel translation, float32, at
3840x2160 (33 MB a frame). Four (prev, next, out) sets rotate, 398 MB together, more than the 129 MB
L2, so each step reads its frames from HBM.

Algorithmic bytes per pixel: harris reads the frame and writes the response (8 B); the corner steps
read the response twice (count, emit: 8 B); the warp reads the frame and writes the output (8 B).
The flow step is a per-feature loop (10 iterations over a 15x15 window, 5 loads a tap, mostly from
L1/L2), reported as features per second.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .stabilize import Stabilizer


def frames(h: int, w: int, shift=(3, -2), seed: int = 0):
    """(prev, next) float32 textures: next shows prev's content moved by shift (dx, dy)."""
    rng = np.random.default_rng(seed)
    m = max(abs(shift[0]), abs(shift[1])) + 8
    # smooth texture: noise upsampled bilinearly from a coarse grid (fast at 4K)
    gh, gw = (h + 2 * m) // 6 + 2, (w + 2 * m) // 6 + 2
    g = rng.random((gh, gw)).astype(np.float32) * 255.0
    ys = np.arange(h + 2 * m, dtype=np.float32) / 6.0
    xs = np.arange(w + 2 * m, dtype=np.float32) / 6.0
    y0, x0 = ys.astype(np.int64), xs.astype(np.int64)
    fy, fx = (ys - y0)[:, None], (xs - x0)[None, :]
    a = g[y0][:, x0]
    b = g[y0][:, x0 + 1]
    c = g[y0 + 1][:, x0]
    d = g[y0 + 1][:, x0 + 1]
    big = (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy
    big = big.astype(np.float32)
    dx, dy = shift
    prev = np.ascontiguousarray(big[m:m + h, m:m + w])
    nxt = np.ascontiguousarray(big[m - dy:m - dy + h, m - dx:m - dx + w])
    return prev, nxt


def run(device, peak_gbs: float, steps: int = 20, warmup: int = 3, h: int = 2160, w: int = 3840) -> dict:
    import torch

    prev, nxt = frames(h, w)
    sets = []
    for i in range(4):
        p = torch.from_numpy(np.roll(prev, i, axis=1)).to(device)
        n = torch.from_numpy(np.roll(nxt, i, axis=1)).to(device)
        sets.append((p, n, torch.empty_like(p)))
    st = Stabilizer(w, h)
    stream = torch.cuda.Stream(device)
    sp = C.c_void_p(stream.cuda_stream)
    L = _lib.lib()
    k, thr, win = 0.04, 1e6, 15

    def check(s):
        if s.code:
            raise RuntimeError(s.message.decode())

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(steps)]
    for i in range(warmup + steps):
        p, n, o = sets[i % len(sets)]
        pp, np_, op = C.c_void_p(p.data_ptr()), C.c_void_p(n.data_ptr()), C.c_void_p(o.data_ptr())
        e = ev[i - warmup] if i >= warmup else None
        if e:
            e[0].record(stream)
        check(L.hmp_stabilizer_corners(st._h, pp, k, thr, sp))
        if e:
            e[1].record(stream)
        check(L.hmp_stabilizer_flow(st._h, pp, np_, win, sp))
        if e:
            e[2].record(stream)
        check(L.hmp_stabilizer_warp(st._h, np_, op, sp))
        if e:
            e[3].record(stream)
    torch.cuda.synchronize(device)
    corners_ms = sum(e[0].elapsed_time(e[1]) for e in ev) / steps
    flow_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / steps
    warp_ms = sum(e[2].elapsed_time(e[3]) for e in ev) / steps
    frame_ms = sum(e[0].elapsed_time(e[3]) for e in ev) / steps
    _, _, motion = st.features(stream)
    px = h * w
    peak = peak_gbs * 1e9
    # end to end: pinned host frames in, the stabilised frame and the motion out, every step
    hp = torch.from_numpy(prev).pin_memory()
    hn = torch.from_numpy(nxt).pin_memory()
    ho = torch.empty_like(hp).pin_memory()
    p, n, o = sets[0]
    info = _lib.StabilizeInfo()
    e2e_steps = max(3, steps // 2)
    torch.cuda.synchronize(device)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(e2e_steps + 1):
        if i == 1:
            t0.record(stream)
        with torch.cuda.stream(stream):
            p.copy_(hp, non_blocking=True)
            n.copy_(hn, non_blocking=True)
        check(L.hmp_stabilizer_run(st._h, C.c_void_p(p.data_ptr()), C.c_void_p(n.data_ptr()),
                                   C.c_void_p(o.data_ptr()), k, thr, win, sp))
        with torch.cuda.stream(stream):
            ho.copy_(o, non_blocking=True)
        check(L.hmp_stabilizer_get_features(st._h, None, None, 0, C.byref(info), sp))  # waits for the stream
    t1.record(stream)
    torch.cuda.synchronize(device)
    e2e_ms = t0.elapsed_time(t1) / e2e_steps
    st.close()
    return {
        "workload": f"stabilize {w}x{h} float32 frame pair, k 0.04, threshold 1e6, window 15",
        "frames": "seeded smooth texture moved by (3, -2); 4 rotating sets > L2",
        "ms_per_frame": round(frame_ms, 4),
        "fps": round(1e3 / frame_ms, 1),
        "corners_ms": round(corners_ms, 4),
        "flow_ms": round(flow_ms, 4),
        "warp_ms": round(warp_ms, 4),
        "features": motion.kept,
        "features_per_s": round(motion.kept / (flow_ms / 1e3), 0),
        "motion": [motion.dx, motion.dy],
        "corners_hbm_frac": round(16.0 * px / (corners_ms / 1e3) / peak, 4),
        "warp_hbm_frac": round(8.0 * px / (warp_ms / 1e3) / peak, 4),
        "e2e_ms_per_frame": round(e2e_ms, 4),
        "e2e_h2d_bytes": 2 * 4 * px,
        "e2e_d2h_bytes": 4 * px + 24,
        "steps": steps,
    }


if __name__ == "__main__":
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser(description="Stabiliser step timings on one GPU.")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--peak-gbs", type=float, default=6695.8)
    a = ap.parse_args()
    print(json.dumps(run(torch.device("cuda", 0), a.peak_gbs, a.steps, a.warmup, a.height, a.width)), flush=True)
