"""The oracle against the reference's golden vectors (CPU).

golden.npz holds stitches produced by the reference's own implementation (its Python port; see
tests/golden/make_golden.py). The oracle is the checker for the CUDA path, so it must reproduce
every case bit for bit before any GPU result is compared with it.
"""
from __future__ import annotations

import numpy as np
import pytest


def _cases(golden):
    return [str(n) for n in golden["names"]]


def test_golden_has_cases(golden):
    names = _cases(golden)
    assert len(names) >= 15
    kinds = {int(golden[f"{n}/meta"][0]) for n in names}
    levels = {int(golden[f"{n}/meta"][2]) for n in names}
    assert kinds == {1, 2}
    assert {0, 1}.issubset(levels) and max(levels) >= 5


def test_oracle_matches_reference_stitches(golden, oracle_lib):
    for name in _cases(golden):
        c = oracle_lib.load_golden_case(golden, name)
        st = oracle_lib.Stitch(c["kind"], c["map_x"], c["map_y"], c["pos_x"], c["pos_y"], c["seam"], c["levels"],
                               c["batch"], c["minimize"])
        out = st.run(c["frames"])
        assert out.shape == c["canvas"].shape, name
        assert np.array_equal(out, c["canvas"]), name


def test_oracle_alpha_renormalised_laplacian(golden, oracle_lib):
    # Known answer of the reference (tests/python/test_pytorch_pano.py:192-201): only the
    # bottom-right low-res tap is valid, so the upsample is that pixel, not a quarter of it.
    lap = oracle_lib.laplacian_rgba(golden["op_laplacian/high"][0], golden["op_laplacian/low"][0])
    assert np.array_equal(lap, golden["op_laplacian/lap"][0])
    assert np.allclose(lap[1, 1, :3], [-100.0, -110.0, -120.0])
    assert lap[1, 1, 3] == 0.0


@pytest.mark.parametrize("op", ["down", "lap", "rec", "mask"])
def test_oracle_pyramid_ops_match_reference(golden, oracle_lib, op):
    img = golden["op_pyr/img"][0]
    down = golden["op_pyr/down"][0]
    if op == "down":
        assert np.array_equal(oracle_lib.downsample_rgba(img), down)
    elif op == "lap":
        assert np.array_equal(oracle_lib.laplacian_rgba(img, down), golden["op_pyr/lap"][0])
    elif op == "rec":
        assert np.array_equal(oracle_lib.reconstruct_rgba(down, golden["op_pyr/lap"][0]), golden["op_pyr/rec"][0])
    else:
        assert np.array_equal(oracle_lib.downsample_mask(golden["op_pyr/mask"]), golden["op_pyr/mask_down"])


def test_oracle_f64_close_to_f32(golden, oracle_lib):
    # The FP64 build differs from the FP32 reference arithmetic by at most one truncation step.
    for name in ["pano2_l6_odd", "panon4_l5_min_b2", "kat_pano2_pattern_l4_min"]:
        c = oracle_lib.load_golden_case(golden, name)
        st = oracle_lib.Stitch(c["kind"], c["map_x"], c["map_y"], c["pos_x"], c["pos_y"], c["seam"], c["levels"],
                               c["batch"], c["minimize"])
        d = np.abs(st.run(c["frames"], "f64").astype(int) - c["canvas"].astype(int))
        assert d.max() <= 1, name


def test_oracle_known_answers(golden, oracle_lib):
    # Hard seam selection (test_pytorch_pano.py:109-128): image 1 left of column 192, image 2 after.
    c = oracle_lib.load_golden_case(golden, "kat_pano2_select_l0")
    out = c["canvas"][0]
    assert (out[:, :192] == [10, 20, 30, 255]).all() and (out[:, 192:] == [100, 110, 120, 255]).all()
    # N hard seam indexed selection (test_pytorch_pano.py:223-246).
    c = oracle_lib.load_golden_case(golden, "kat_panon3_select_l0")
    out = c["canvas"][0]
    assert (out[:, :16] == [10, 0, 0, 255]).all()
    assert (out[:, 16:32] == [0, 20, 0, 255]).all()
    assert (out[:, 32:] == [0, 0, 30, 255]).all()
    # minimize == full (test_pytorch_pano.py:155-189, 204-220).
    for a, b in [("kat_pano2_pattern_l4_min", "kat_pano2_pattern_l4_full"),
                 ("kat_panon2_pattern_l4_min", "kat_panon2_pattern_l4_full")]:
        assert np.array_equal(golden[f"{a}/canvas"], golden[f"{b}/canvas"])


def _px(*v):
    return np.array(v, np.float32).reshape(1, 1, -1)


def test_oracle_nway_blend_known_answers(oracle_lib):
    """The reference's N-way blend tests (src/cuda/cudaBlendN_test.cpp:27-183), through the
    oracle's whole Laplacian blend with a float mask (one weight per image), tolerance 1e-5 as there."""
    o = oracle_lib
    # An alpha-0 image drops out and the weights renormalise: 0.1/0.8/0.1 -> 0.5/0/0.5 (:27-70).
    out = o.laplacian_blend([_px(10, 20, 30, 255), _px(100, 110, 120, 0), _px(90, 100, 110, 255)],
                            _px(0.1, 0.8, 0.1), 1, o.RULE_NWAY)
    np.testing.assert_allclose(out[0, 0], [50, 60, 70, 255], atol=1e-5)
    # Four levels of constant images with weights 0.25 / 0.75 give the weighted mean everywhere (:73-139).
    i0 = np.tile(np.array([10, 20, 30, 255], np.float32), (8, 8, 1))
    i1 = np.tile(np.array([110, 120, 130, 255], np.float32), (8, 8, 1))
    m = np.tile(np.array([0.25, 0.75], np.float32), (8, 8, 1))
    out = o.laplacian_blend([i0, i1], m, 4, o.RULE_NWAY)
    np.testing.assert_allclose(out.reshape(-1, 4), np.tile([85, 95, 105, 255], (64, 1)), atol=1e-5)
    # The mask selects only a transparent image: the highest-alpha image is copied (:142-183).
    out = o.laplacian_blend([_px(255, 0, 0, 255), _px(0, 255, 0, 0), _px(0, 0, 255, 128)], _px(0, 1, 0), 1,
                            o.RULE_NWAY)
    np.testing.assert_allclose(out[0, 0], [255, 0, 0, 255], atol=1e-5)


def test_oracle_three_image_blend_known_answers(oracle_lib):
    """The reference's three-image blend tests (src/cuda/cudaBlend3_test.cpp:62-387), through the
    oracle's three-image rule, tolerance 1e-5 as there."""
    o = oracle_lib
    rgb = [_px(10, 20, 30), _px(40, 50, 60), _px(70, 80, 90)]
    # One-hot masks pick one RGB image (:62-150).
    for k in range(3):
        w = [0.0, 0.0, 0.0]
        w[k] = 1.0
        np.testing.assert_allclose(o.laplacian_blend(rgb, _px(*w), 1, o.RULE_THREE)[0, 0], rgb[k][0, 0], atol=1e-5)
    # Equal weights of 1, 2, 3 give 2 (:152-196).
    out = o.laplacian_blend([np.full((2, 2, 3), v, np.float32) for v in (1, 2, 3)],
                            np.full((2, 2, 3), 1 / 3, np.float32), 1, o.RULE_THREE)
    np.testing.assert_allclose(out, 2.0, atol=1e-5)
    # RGBA: colour weighted 0.2 / 0.3 / 0.5, alpha the largest (:198-248).
    out = o.laplacian_blend([_px(10, 20, 30, 40), _px(50, 60, 70, 80), _px(90, 100, 110, 120)], _px(0.2, 0.3, 0.5), 1,
                            o.RULE_THREE)
    np.testing.assert_allclose(out[0, 0], [62, 72, 82, 120], atol=1e-5)
    # An alpha-0 image drops out (:255-289) and a mask on a transparent image falls back (:291-328).
    out = o.laplacian_blend([_px(10, 20, 30, 255), _px(100, 110, 120, 0), _px(90, 100, 110, 255)],
                            _px(0.1, 0.8, 0.1), 1, o.RULE_THREE)
    np.testing.assert_allclose(out[0, 0], [50, 60, 70, 255], atol=1e-5)
    out = o.laplacian_blend([_px(255, 0, 0, 255), _px(0, 255, 0, 0), _px(0, 0, 255, 128)], _px(0, 1, 0), 1,
                            o.RULE_THREE)
    np.testing.assert_allclose(out[0, 0], [255, 0, 0, 255], atol=1e-5)
    # Two levels across a top/bottom seam leave no alpha holes and no vanished colour (:330-387).
    imgs = []
    for c, v in ((0, 100), (1, 150), (2, 200)):
        a = np.zeros((4, 4, 4), np.float32)
        a[..., c] = v
        a[..., 3] = 255
        imgs.append(a)
    m = np.zeros((4, 4, 3), np.float32)
    m[:2, :, 0] = 1
    m[2:, :, 1] = 1
    out = o.laplacian_blend(imgs, m, 2, o.RULE_THREE)
    for y in (1, 2):
        assert (out[y, :, 3] >= 250).all() and (out[y, :, :3].sum(axis=-1) > 50).all()


@pytest.mark.parametrize("name", ["two_way_overlap", "no_overlap", "gap", "multi_seam_intersection"])
def test_oracle_reference_pano_layouts(oracle_lib, name):
    """The reference's N-image stitcher tests (src/pano/cudaPanoN_test.cpp:192-298) on the oracle:
    the minimised blend equals the full-canvas blend (there within 1e-4 on float pixels; here the
    uint8 canvases are equal), and an uncovered gap stays transparent."""
    import pano_layouts as pl

    lay = pl.layouts()[name]
    mx, my = pl.tables(lay)
    px, py = zip(*lay["positions"])
    fr = pl.frames(lay)
    outs = [oracle_lib.Stitch(pl.KIND_PANON, mx, my, px, py, lay["seam"], lay["levels"], 1, minimize).run(fr)
            for minimize in (False, True)]
    assert np.array_equal(outs[0], outs[1]), name
    if lay["gap"]:
        x0, x1 = lay["gap"]
        assert (outs[1][0, :, x0:x1, 3] == 0).all()
        assert (outs[1][0, :, :x0, 3] == 255).all() and (outs[1][0, :, x1:, 3] == 255).all()


def test_oracle_three_image_trivial_stitches(oracle_lib):
    """The reference's three-image stitcher tests (src/pano/cudaPano3_test.cpp:56-196) on a 1x1
    canvas with all three tables at (0, 0): label 2 under the hard seam takes the third (RGB)
    image; label 1 with one level takes the middle image, alpha kept."""
    z = [np.zeros((1, 1), np.uint16)] * 3
    st = oracle_lib.Stitch(3, z, z, [0, 0, 0], [0, 0, 0], np.array([[2]], np.uint8), 0)
    out = st.run([np.full((1, 1, 1, 3), v, np.uint8) for v in (10, 50, 200)])
    assert (st.canvas_w, st.canvas_h) == (1, 1) and out[0, 0, 0].tolist() == [200, 200, 200]
    frames = []
    for v in (30, 60, 90):
        f = np.full((1, 1, 1, 4), v, np.uint8)
        f[..., 3] = 255
        frames.append(f)
    out = oracle_lib.Stitch(3, z, z, [0, 0, 0], [0, 0, 0], np.array([[1]], np.uint8), 1).run(frames)
    assert out[0, 0, 0].tolist() == [60, 60, 60, 255]
