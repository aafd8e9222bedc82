"""Frame times of the named workloads besides the headline frame, each alone on one stream.

* the two-image production frame (2 x 5120x2880 -> 8500x3300) at 6 levels with FP16 level
  storage, with the 5-tap Binomial5 filter, and as a hard seam (0 levels);
* the eight-image rig (8 x 2000x1500 -> 9000x2400, 45-degree steps) at 6 levels, FP32 and FP16;
* the three-image stream of the batched workload (3 x 2704x1520 -> 6000x1800) at 6 levels, FP32
  and FP16;
* the headline frame with copy blocks for frames promised opaque (no per-call alpha check and no
  fallback launch).

Each variant: one stitcher, batch 1, two rotating frame/canvas sets (every set is larger than the
129 MB L2), warm-up calls, then CUDA events around `steps` process() calls on one stream.
Reported: ms per frame, fps, canvas Mpix/s and the frame's compulsory bytes (M0, the stitcher's
own count: tables, seam, source and canvas pixels) over its time as a fraction of the measured
copy bandwidth.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib, pano, synth

VARIANTS = [
    # (name, workload, kind, levels, storage, filter)
    ("pano2_l6_f32", "pano2_5120x2880_to_8500x3300", 2, 6, "f32", "refbox"),
    ("pano2_l6_f16", "pano2_5120x2880_to_8500x3300", 2, 6, "f16", "refbox"),
    ("pano2_l6_binomial5", "pano2_5120x2880_to_8500x3300", 2, 6, "f32", "binomial5"),
    ("pano2_l0", "pano2_5120x2880_to_8500x3300", 2, 0, "f32", "refbox"),
    ("panon8_l6_f32", "panon8_2000x1500_to_9000x2400", 1, 6, "f32", "refbox"),
    ("panon8_l6_f16", "panon8_2000x1500_to_9000x2400", 1, 6, "f16", "refbox"),
    ("pano3_l6_f32", "pano3_2704x1520_to_6000x1800", 3, 6, "f32", "refbox"),
    ("pano3_l6_f16", "pano3_2704x1520_to_6000x1800", 3, 6, "f16", "refbox"),
    ("pano2_l6_f32_opaque", "pano2_5120x2880_to_8500x3300", 2, 6, "f32", "refbox"),
]
# Variants run with copy blocks for frames promised opaque (hmp_stitcher_set_copy_blocks mode 2:
# no per-call alpha check, no fallback launch); the synthetic frames are opaque (alpha 255).
OPAQUE = {"pano2_l6_f32_opaque"}


def masks_for(kind: int, rig):
    pos = [pano.SpatialTiff(float(x), float(y)) for x, y in zip(rig.pos_x, rig.pos_y)]
    if kind == 2:
        return pano.ControlMasks(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.seam, pos)
    if kind == 3:
        return pano.ControlMasks3(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.map_x[2], rig.map_y[2],
                                  rig.seam, pos)
    return pano.ControlMasksN(list(rig.map_x), list(rig.map_y), rig.seam, pos)


def stitcher(kind: int, masks, levels: int, **kw):
    if kind == 2:
        return pano.CudaStitchPano(1, levels, masks, quiet=True, **kw)
    if kind == 3:
        return pano.CudaStitchPano3(1, levels, masks, quiet=True, **kw)
    return pano.CudaStitchPanoN(1, levels, masks, quiet=True, **kw)


def time_frames(st, sets, steps: int, warmup: int, device) -> float:
    """Milliseconds per process() over `steps` calls rotating through `sets` (CUDA events)."""
    import torch

    stream = torch.cuda.Stream(device)
    sp = C.c_void_p(stream.cuda_stream)
    fn = _lib.lib().hmp_stitcher_process
    calls = [((_lib.Image * len(ins))(*[pano._image(t) for t in ins]), len(ins), pano._image(cv)) for ins, cv in sets]

    def go(k):
        for j in range(k):
            imgs, n, cv = calls[j % len(calls)]
            s = fn(st._handle, imgs, n, C.byref(cv), sp)
            if s.code:
                raise RuntimeError(s.message.decode())

    go(warmup)
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    go(steps)
    e1.record(stream)
    torch.cuda.synchronize(device)
    return e0.elapsed_time(e1) / steps


def run(device, steps: int, peak_gbs: float, warmup: int = 5, only=None) -> dict:
    import torch

    rigs = {}
    out = {}
    for name, workload, kind, levels, storage, filt in VARIANTS:
        if only and name not in only:
            continue
        if workload not in rigs:
            rig = synth.workload_rig(workload, seed=1234, kind=kind)
            host = synth.rig_frames(rig, seed=1)
            sets = []
            for i in range(2):
                ins = [torch.from_numpy(np.roll(f, i, axis=2)).to(device) for f in host]
                sets.append((ins, torch.empty((1, rig.canvas_h, rig.canvas_w, 4), dtype=torch.uint8, device=device)))
            rigs[workload] = (rig, sets, masks_for(kind, rig))
        rig, sets, masks = rigs[workload]
        st = stitcher(kind, masks, levels, storage=storage, filter=filt)
        if not st.status.ok():
            raise pano.CudaStatusError(st.status)
        if name in OPAQUE:
            st.set_copy_blocks(True, opaque_frames=True)
        ms = time_frames(st, sets, steps, warmup, device)
        info = st.info()
        mpix = rig.canvas_w * rig.canvas_h / 1e6
        out[name] = {"workload": workload, "levels": levels, "storage": storage, "filter": filt,
                     "copy_blocks": "opaque frames" if name in OPAQUE else "checked",
                     "ms_per_frame": round(ms, 5), "fps": round(1e3 / ms, 1), "mpix_s": round(mpix / ms * 1e3, 1),
                     "m0_bytes": int(info["m0_bytes"]),
                     "hbm_frac_frame": round(info["m0_bytes"] / (ms / 1e3) / (peak_gbs * 1e9), 4),
                     "launches_per_frame": int(info["launches_per_process"]), "steps": steps}
        del st
    torch.cuda.synchronize(device)
    return out


if __name__ == "__main__":
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser(description="Frame times of the named workloads (one stitcher each, one stream).")
    ap.add_argument("--only", default="", help="comma-separated variant names (default: all): "
                    + ", ".join(v[0] for v in VARIANTS))
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--peak-gbs", type=float, default=6695.8, help="copy bandwidth for hbm_frac_frame")
    args = ap.parse_args()
    only = [s for s in args.only.split(",") if s] or None
    for name, res in run(torch.device("cuda", 0), args.steps, args.peak_gbs, args.warmup, only).items():
        print(json.dumps({"variant": name, **res}), flush=True)
