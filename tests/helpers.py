"""Shared helpers for the tests: turn golden cases and synthetic rigs into stitcher inputs."""
from __future__ import annotations

import numpy as np

from hmpano import synth


def masks_for(kind: int, map_x, map_y, pos_x, pos_y, seam):
    import hmpano

    pos = [hmpano.SpatialTiff(float(x), float(y)) for x, y in zip(pos_x, pos_y)]
    if kind == 2:
        m = hmpano.ControlMasks()
        m.img1_col, m.img1_row, m.img2_col, m.img2_row = map_x[0], map_y[0], map_x[1], map_y[1]
        m.whole_seam_mask_image = seam
    elif kind == 3:
        m = hmpano.ControlMasks3()
        m.img0_col, m.img0_row = map_x[0], map_y[0]
        m.img1_col, m.img1_row = map_x[1], map_y[1]
        m.img2_col, m.img2_row = map_x[2], map_y[2]
        m.whole_seam_mask_image = seam
    else:
        m = hmpano.ControlMasksN()
        m.img_col, m.img_row = list(map_x), list(map_y)
        m.whole_seam_mask_indexed = seam
    m.positions = pos
    return m


def masks_for_case(c):
    return masks_for(c["kind"], c["map_x"], c["map_y"], c["pos_x"], c["pos_y"], c["seam"])


def masks_for_rig(rig: synth.Rig):
    return masks_for(rig.kind, rig.map_x, rig.map_y, rig.pos_x, rig.pos_y, rig.seam)


def make_stitcher(kind: int, masks, levels: int, batch: int = 1, minimize: bool = True, **kw):
    import hmpano

    if kind == 2:
        return hmpano.CudaStitchPano(batch, levels, masks, quiet=True, minimize_blend=minimize, **kw)
    if kind == 3:
        return hmpano.CudaStitchPano3(batch, levels, masks, quiet=True, **kw)
    return hmpano.CudaStitchPanoN(batch, levels, masks, quiet=True, minimize_blend=minimize, **kw)


def gpu_stitch(stitcher, frames, canvas=None):
    """Run one process() on CUDA tensors made from numpy frames; returns the canvas as numpy."""
    import torch

    ins = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in frames]
    out = stitcher._run(ins, canvas)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def lsb_stats(a: np.ndarray, b: np.ndarray) -> tuple[int, float]:
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return int(d.max()), float(d.mean())
