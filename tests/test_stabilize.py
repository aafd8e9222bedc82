"""The frame stabiliser on the CPU: the oracle (oracle/hmp_stabilize_oracle.c) against an
independent numpy restatement of src/cuda/cudaStabilize.cu, its tracking on known translations,
and the C ABI's argument checks (no device work).

The reference ships the stabiliser as a demo program with no tests or vectors, so its parity is
unpinned; the numpy restatement below follows the reference kernels line by line in float32
(every numpy float32 operation rounds once, like the reference without fused multiply-add).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from stab_frames import moving_pair, texture


def np_harris(img: np.ndarray, k: float) -> np.ndarray:
    """computeGradients + computeHarrisResponse (cudaStabilize.cu:24-69), undefined borders = 0."""
    f = np.float32
    h, w = img.shape
    gx = np.zeros((h, w), f)
    gy = np.zeros((h, w), f)
    r0, r1, r2 = img[:-2], img[1:-1], img[2:]
    gx[1:-1, 1:-1] = (r0[:, 2:] + f(2.0) * r1[:, 2:] + r2[:, 2:] - r0[:, :-2] - f(2.0) * r1[:, :-2] - r2[:, :-2])
    gy[1:-1, 1:-1] = (r0[:, :-2] + f(2.0) * r0[:, 1:-1] + r0[:, 2:] - r2[:, :-2] - f(2.0) * r2[:, 1:-1] - r2[:, 2:])
    sxx = np.zeros((h - 2, w - 2), f)
    sxy = np.zeros((h - 2, w - 2), f)
    syy = np.zeros((h - 2, w - 2), f)
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            ix = gx[1 + j:h - 1 + j, 1 + i:w - 1 + i]
            iy = gy[1 + j:h - 1 + j, 1 + i:w - 1 + i]
            sxx = sxx + ix * ix
            sxy = sxy + ix * iy
            syy = syy + iy * iy
    det = sxx * syy - sxy * sxy
    tr = sxx + syy
    resp = np.zeros((h, w), f)
    resp[1:-1, 1:-1] = det - f(k) * tr * tr
    return resp


def np_corners(resp: np.ndarray, thr: float) -> np.ndarray:
    """Threshold + 3x3 non-maximum suppression, raster order (cudaStabilize.cu:179-199)."""
    h, w = resp.shape
    c = resp[1:-1, 1:-1]
    keep = c > np.float32(thr)
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            keep &= ~(resp[1 + j:h - 1 + j, 1 + i:w - 1 + i] > c)
    ys, xs = np.nonzero(keep)
    return np.stack([xs + 1, ys + 1], 1).astype(np.int32)


@pytest.mark.parametrize("h,w", [(3, 3), (23, 37), (120, 161)])
def test_oracle_harris_and_corners_match_numpy_restatement(oracle_lib, h, w):
    prev, nxt = moving_pair(h, w, (1, -1), seed=h)
    for k, thr in [(0.04, 1e6), (0.06, 0.0), (0.04, -1e30)]:
        r = oracle_lib.Stabilize(k=k, threshold=thr).run(prev, nxt)
        resp = np_harris(prev, k)
        assert np.array_equal(r["response"], resp)
        assert np.array_equal(r["corners"], np_corners(resp, thr).reshape(-1, 2))
        assert r["found"] == len(r["corners"])


def np_flow(prev, nxt, xy, window):
    """lucasKanadeOpticalFlowKernel (cudaStabilize.cu:75-131) for one feature at a time, float32,
    taps in column 0 / row 0 skipped."""
    f = np.float32
    h, w = prev.shape
    half = window // 2
    out = np.zeros((len(xy), 2), f)
    for n, (px, py) in enumerate(xy):
        dx = dy = f(0.0)
        for _ in range(10):
            s = [f(0.0)] * 5
            rdx, rdy = int(np.round(dx)), int(np.round(dy))
            for j in range(-half, half + 1):
                for i in range(-half, half + 1):
                    x, y = px + i, py + j
                    xn, yn = x + rdx, y + rdy
                    if x < 1 or x >= w - 1 or y < 1 or y >= h - 1 or xn < 0 or xn >= w - 1 or yn < 0 or yn >= h - 1:
                        continue
                    ix = (prev[y, x + 1] - prev[y, x - 1]) * f(0.5)
                    iy = (prev[y + 1, x] - prev[y - 1, x]) * f(0.5)
                    it = nxt[yn, xn] - prev[y, x]
                    s = [s[0] + ix * ix, s[1] + iy * iy, s[2] + ix * iy, s[3] + ix * it, s[4] + iy * it]
            det = s[0] * s[1] - s[2] * s[2]
            if abs(det) < f(1e-6):
                break
            ddx = (-s[1] * s[3] + s[2] * s[4]) / det
            ddy = (s[2] * s[3] - s[0] * s[4]) / det
            dx, dy = f(dx + ddx), f(dy + ddy)
            if np.sqrt(f(ddx * ddx + ddy * ddy)) < f(0.01):
                break
        out[n] = (dx, dy)
    return out


def test_oracle_flow_matches_numpy_restatement(oracle_lib):
    prev, nxt = moving_pair(40, 56, (2, -1), seed=5)
    feats = np.array([[0, 0], [1, 1], [20, 17], [55, 39], [3, 30], [54, 2], [28, 20]], np.int32)
    with np.errstate(all="ignore"):
        want = np_flow(prev, nxt, feats, 7)
    r = oracle_lib.Stabilize(window=7).run(prev, nxt, features=feats)
    assert np.array_equal(r["flow"], want)


@pytest.mark.parametrize("shift", [(-3, 2), (1, 0), (0, -2), (4, 3)])
def test_oracle_tracks_a_known_translation(oracle_lib, shift):
    prev, nxt = moving_pair(240, 320, shift, seed=3)
    r = oracle_lib.Stabilize().run(prev, nxt)
    assert r["found"] > 500
    assert (round(r["dx"]), round(r["dy"])) == shift
    med = np.median(r["flow"], 0)
    assert abs(med[0] - shift[0]) < 0.35 and abs(med[1] - shift[1]) < 0.35  # one-level LK on integer taps
    # the reference's warp samples next at (x - shift_x, y - shift_y)
    sx, sy = shift
    out = r["out"]
    h, w = nxt.shape
    want = np.zeros_like(nxt)
    want[max(sy, 0):h + min(sy, 0), max(sx, 0):w + min(sx, 0)] = nxt[max(-sy, 0):h - max(sy, 0),
                                                                     max(-sx, 0):w - max(sx, 0)]
    assert np.array_equal(out, want)


def test_oracle_without_corners_does_not_move(oracle_lib):
    prev = np.full((30, 40), 7.0, np.float32)  # flat: zero response everywhere
    nxt = texture(30, 40, seed=1)
    r = oracle_lib.Stabilize().run(prev, nxt)
    assert r["found"] == 0 and r["dx"] == 0.0 and r["dy"] == 0.0
    assert np.array_equal(r["out"], nxt)


def test_oracle_feature_cap_tracks_the_first_corners(oracle_lib):
    prev, nxt = moving_pair(120, 160, (2, 1), seed=4)
    full = oracle_lib.Stabilize().run(prev, nxt)
    capped = oracle_lib.Stabilize(max_features=10).run(prev, nxt)
    assert capped["found"] == full["found"] > 10
    assert np.array_equal(capped["corners"], full["corners"][:10])
    assert np.array_equal(capped["flow"], full["flow"][:10])


def test_stabilizer_abi_rejects_bad_arguments_before_any_device_work():
    from hmpano import _lib

    lib = _lib.lib()
    h = C.c_void_p()
    for w_, h_, m in [(2, 10, 0), (10, 2, 0), (40000, 10, 0), (10, 10, -1)]:
        s = lib.hmp_stabilizer_create(w_, h_, m, C.byref(h))
        assert s.code == 1 and not h.value, (w_, h_, m, s.message)
    assert lib.hmp_stabilizer_create(10, 10, 0, None).code == 1
    assert lib.hmp_stabilizer_corners(None, None, 0.04, 1e6, None).code == 1
    assert lib.hmp_stabilizer_flow(None, None, None, 15, None).code == 1
    assert lib.hmp_stabilizer_warp(None, None, None, None).code == 1
    assert lib.hmp_stabilizer_run(None, None, None, None, 0.04, 1e6, 15, None).code == 1
    info = _lib.StabilizeInfo()
    assert lib.hmp_stabilizer_get_features(None, None, None, 0, C.byref(info), None).code == 1
    assert lib.hmp_stabilizer_get_response(None, None, 0, None).code == 1
    assert lib.hmp_stabilizer_set_features(None, None, 0, None).code == 1
    lib.hmp_stabilizer_destroy(None)


def test_oracle_warp_rounds_extreme_motion_like_the_gpu(oracle_lib):
    """The warp's shift is the motion rounded as the GPU's float-to-int conversion does it:
    NaN shifts nothing, a shift past the frame leaves only zero fill (clamped at 2^24)."""
    from oracle.oracle import _ptr
    import ctypes as C

    L = oracle_lib.lib()
    img = texture(20, 30, seed=3)
    out = np.full_like(img, -1.0)
    for dx, dy, want in [(float("nan"), 0.0, img), (0.0, float("nan"), img),
                         (1e30, 0.0, np.zeros_like(img)), (-1e30, 2.0, np.zeros_like(img)),
                         (0.4, -0.4, img)]:
        L.hmpo_stab_warp(_ptr(img, C.c_float), 30, 20, dx, dy, _ptr(out, C.c_float))
        assert np.array_equal(out, want), (dx, dy)
