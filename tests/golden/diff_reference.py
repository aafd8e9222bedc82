"""Differential check of the oracle against the reference's own Python implementation on random
rigs (beyond the fixed golden cases).

Like make_golden.py it imports hm-cupano's ``cupano`` package with stand-in cv2/tifffile/PIL
modules and the workspace-downsample correction, so it needs the reference tree; the tests do not
run it. Each rig draws 2 to --max-images (default 5, at most 8) images, canvas and source sizes,
overlap, levels 0..6, minimised or full blend, batch 1 or 2, out-of-range table entries and RGB
or RGBA frames, runs the reference and the FP32 oracle, and compares the canvases bit for bit.

Two kinds of rig are left out because the two implementations are known to differ there:
  * two images under the N-image stitcher at levels > 0 (the Python CudaStitchPanoN uses the
    two-image rule, the C++ one the N-way rule, which this build follows);
  * configurations the oracle rejects, counted as "rejected" without running the reference (it
    rejects some of them too; others it accepts, such as a minimised two-image strip that leaves
    the canvas, which this build rejects).

Usage: python tests/golden/diff_reference.py [--seed S] [--rigs N] [--reference /path/to/hm-cupano]
Prints one line per differing rig and a summary; exit status 1 if any canvas differs.
"""
from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path[:0] = [str(HERE), str(REPO), str(REPO / "hm-cupano_gb300")]

import make_golden as mg  # noqa: E402
from hmpano import synth  # noqa: E402


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--rigs", type=int, default=100)
    ap.add_argument("--max-images", type=int, default=5, help="images per rig: 2..max (at most 8)")
    ap.add_argument("--reference", default=os.environ.get("HM_CUPANO_REFERENCE"),
                    required="HM_CUPANO_REFERENCE" not in os.environ,
                    help="the hm-cupano checkout (default: $HM_CUPANO_REFERENCE)")
    args = ap.parse_args()
    mg._install_stubs()
    sys.path.insert(0, args.reference)
    import torch

    torch.set_num_threads(max(1, os.cpu_count() or 1))
    import cupano
    from cupano import ops as ref_ops

    from oracle import oracle

    mg.install_corrections(ref_ops)
    oracle.build()
    rng = np.random.default_rng(args.seed)
    same = differ = rejected = 0
    for t in range(args.rigs):
        n = int(rng.choice([2, 2] + list(range(3, min(args.max_images, 8) + 1))))
        kind = 2 if n == 2 else 1
        params = dict(canvas_w=int(rng.integers(300, 700)), canvas_h=int(rng.integers(16, 64)), n=n,
                      src_w=int(rng.integers(100, 260)), src_h=int(rng.integers(14, 60)),
                      overlap=(int(rng.integers(60, 120)) if kind == 2 else float(rng.uniform(0.2, 0.35))),
                      yaw_step_deg=float(rng.uniform(30, 55)))
        levels = int(rng.integers(0, 7))
        minimize = bool(rng.integers(0, 2))
        batch = int(rng.integers(1, 3))
        oob = float(rng.choice([0.0, 0.0, 0.05]))
        rgb = bool(rng.random() < 0.25)
        rig = synth.make_rig(seed=int(rng.integers(0, 10000)), kind=kind, oob_fraction=oob, **params)
        frames = [synth.make_frame(rig.src_w[i], rig.src_h[i], int(rng.integers(0, 1000)) * 10 + i, batch)
                  for i in range(rig.n)]
        if rgb:
            frames = [f[..., :3].copy() for f in frames]
        try:
            out = oracle.Stitch.from_rig(rig, levels, batch, minimize).run(frames)
        except (ValueError, RuntimeError):
            rejected += 1
            continue
        ref = mg._run_reference(cupano, rig, frames, levels, minimize, batch)
        if out.shape == ref.shape and np.array_equal(out, ref):
            same += 1
            continue
        differ += 1
        if out.shape != ref.shape:
            print(f"rig {t}: shapes {out.shape} vs {ref.shape}")
            continue
        d = np.abs(out.astype(int) - ref.astype(int))
        where = np.argwhere(d > 0)[:3].tolist()
        print(f"rig {t}: kind {kind} n {n} levels {levels} minimize {minimize} batch {batch} rgb {rgb}: "
              f"{int((d > 0).sum())} samples differ, max {int(d.max())} LSB, at {where}")
    print(f"seed {args.seed}: {same} equal, {differ} differ, {rejected} rejected by the oracle")
    return 1 if differ else 0


if __name__ == "__main__":
    sys.exit(main())
