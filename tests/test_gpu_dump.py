"""Soft-blend pyramid dump (hmp_stitcher_dump_pyramid, the reference's dump_soft_blend_pyramid).

Each dumped level is checked, bit for bit, against the oracle's operation applied to the level it
comes from (downsample, Laplacian, two-image blend, reconstruction), and the reconstruction at
level 0, packed, against the canvas the stitcher wrote. Metadata follows the reference test
(src/pano/cudaPano_test.cpp:141-204): level 0 spans the canvas width for the full blend and less
for the minimised one, at the canvas height.
"""
from __future__ import annotations

import struct

import numpy as np
import pytest

from helpers import make_stitcher, masks_for_rig

pytestmark = pytest.mark.gpu


def read_tiff_f32(path) -> np.ndarray:
    """The dump's TIFF layout: little-endian, uncompressed, one strip of float32 samples."""
    b = path.read_bytes()
    assert b[:4] == b"II*\0"
    ifd = struct.unpack_from("<I", b, 4)[0]
    tags = {}
    for i in range(struct.unpack_from("<H", b, ifd)[0]):
        tag, typ, cnt, val = struct.unpack_from("<HHII", b, ifd + 2 + 12 * i)
        tags[tag] = val & 0xFFFF if (typ == 3 and cnt == 1) else val
    w, h, ch = tags[256], tags[257], tags[277]
    assert tags[259] == 1 and tags[284] == 1
    return np.frombuffer(b, dtype="<f4", count=w * h * ch, offset=tags[273]).reshape(h, w, ch)


def pack_u8(v: np.ndarray) -> np.ndarray:
    return np.where(v <= 0, 0, np.where(v >= 255, 255, np.trunc(np.clip(v, 0, 255)))).astype(np.uint8)


def read_metadata(path) -> dict:
    return dict(line.split("=", 1) for line in path.read_text().split())


@pytest.mark.parametrize("minimize", [True, False])
def test_dump_levels_match_oracle_steps_and_canvas(tmp_path, oracle_lib, minimize):
    import torch
    from hmpano import synth

    levels, batch = 4, 2
    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=23, kind=2, scale=0.25)
    frames = synth.rig_frames(rig, seed=3, batch=batch)
    st = make_stitcher(2, masks_for_rig(rig), levels, batch, minimize)
    assert st.status.ok(), st.status
    ins = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in frames]  # kept alive for the dump
    canvas = st._run(ins).cpu().numpy()
    st.dump_soft_blend_pyramid(tmp_path)

    info = st.info()
    bx, by, bw, bh = info["blend_rect"]
    wx, wy, ww, wh = info["write_rect"]
    meta = read_metadata(tmp_path / "metadata.txt")
    L = int(meta["num_levels"])
    assert L == levels and int(meta["batch_size"]) == batch and int(meta["channels"]) == 4
    assert meta["level_0"] == f"{bw}x{bh}"
    assert bh == st.canvas_height()
    if minimize:
        assert bw < st.canvas_width()
    else:
        assert bw == st.canvas_width()

    def lv(label, l, b=None):
        name = f"level_{l}.tiff" if b is None else f"level_{l}_batch_{b}.tiff"
        return read_tiff_f32(tmp_path / label / name)

    masks = [lv("mask", l)[..., 0] for l in range(L)]
    for l in range(L - 1):
        np.testing.assert_array_equal(masks[l + 1], oracle_lib.downsample_mask(masks[l][..., None])[..., 0])
    for b in range(batch):
        g = {k: [lv(k, l, b) for l in range(L)] for k in ("gauss1", "gauss2")}
        lap = {k: [lv(k, l, b) for l in range(L)] for k in ("lap1", "lap2")}
        blend = [lv("blend", l, b) for l in range(L)]
        rec = [lv("reconstruct", l, b) for l in range(L)]
        for gk, lk in (("gauss1", "lap1"), ("gauss2", "lap2")):
            for l in range(L - 1):
                np.testing.assert_array_equal(g[gk][l + 1], oracle_lib.downsample_rgba(g[gk][l]), err_msg=f"{gk} {l + 1}")
                np.testing.assert_array_equal(lap[lk][l], oracle_lib.laplacian_rgba(g[gk][l], g[gk][l + 1]),
                                              err_msg=f"{lk} {l}")
            np.testing.assert_array_equal(lap[lk][L - 1], g[gk][L - 1])
        for l in range(L):
            np.testing.assert_array_equal(blend[l], oracle_lib.blend_two_rgba(lap["lap1"][l], lap["lap2"][l], masks[l]),
                                          err_msg=f"blend {l}")
        np.testing.assert_array_equal(rec[L - 1], blend[L - 1])
        for l in range(L - 1):
            np.testing.assert_array_equal(rec[l], oracle_lib.reconstruct_rgba(rec[l + 1], blend[l]), err_msg=f"rec {l}")
        x0, y0 = wx - bx, wy - by
        np.testing.assert_array_equal(pack_u8(rec[0][y0:y0 + wh, x0:x0 + ww]), canvas[b, wy:wy + wh, wx:wx + ww])


def test_dump_errors(tmp_path):
    from hmpano import pano, synth

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=23, kind=2, scale=0.25)
    fresh = make_stitcher(2, masks_for_rig(rig), 3)
    with pytest.raises(pano.CudaStatusError, match="populated"):
        fresh.dump_soft_blend_pyramid(tmp_path)
    hard = make_stitcher(2, masks_for_rig(rig), 0)
    with pytest.raises(pano.CudaStatusError, match="num_levels > 0"):
        hard.dump_soft_blend_pyramid(tmp_path)
