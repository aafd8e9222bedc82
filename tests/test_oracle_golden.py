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
