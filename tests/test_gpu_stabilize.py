"""The frame stabiliser on the GPU (hmp_stabilizer_*), bit for bit against the oracle
(oracle/hmp_stabilize_oracle.c, a restatement of src/cuda/cudaStabilize.cu): the Harris response
map, the corner list in raster order, every feature's flow, the mean motion and the warped frame.

Sizes run from the smallest frame the stabiliser takes (3 x 3) through ragged tiles to the
reference's demo size (640 x 480) and full HD; cases cover a feature cap, caller-given features
(on the border too), a flat frame with no corners, the in-place warp of the reference, a frame
sequence through one stabiliser and CUDA graph replay.
"""
from __future__ import annotations

import numpy as np
import pytest

from stab_frames import moving_pair, texture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _check(st, ref, out_dev):
    xy, flow, m = st.features()
    assert m.corners == ref["found"], (m.corners, ref["found"])
    assert np.array_equal(st.response(), ref["response"])
    assert np.array_equal(xy, ref["corners"].reshape(-1, 2))
    if not np.array_equal(flow, ref["flow"].reshape(-1, 2)):
        bad = np.argwhere((flow != ref["flow"]).any(1)).ravel()
        pytest.fail(f"flow differs at {len(bad)} features, first {bad[:5].tolist()}: "
                    f"{flow[bad[:3]].tolist()} vs {ref['flow'][bad[:3]].tolist()}")
    assert (m.dx, m.dy) == (ref["dx"], ref["dy"])
    assert (m.shift_x, m.shift_y) == (int(np.round(ref["dx"])), int(np.round(ref["dy"])))
    assert np.array_equal(out_dev.cpu().numpy(), ref["out"])


@pytest.mark.parametrize("h,w,shift", [
    (3, 3, (0, 0)),
    (23, 37, (1, -1)),
    (480, 640, (-3, 2)),
    (479, 641, (5, -4)),
    (1080, 1920, (2, 3)),
])
def test_stabilizer_matches_oracle(oracle_lib, h, w, shift):
    import hmpano

    prev, nxt = moving_pair(h, w, shift, seed=w)
    ref = oracle_lib.Stabilize().run(prev, nxt)
    st = hmpano.Stabilizer(w, h)
    p, n = _dev(prev), _dev(nxt)
    out = _dev(np.full((h, w), -1, np.float32))
    st.run(p, n, out)
    _check(st, ref, out)
    assert np.array_equal(n.cpu().numpy(), nxt)  # next untouched when out is another buffer


@pytest.mark.parametrize("k,thr,window", [(0.06, 0.0, 7), (0.04, 5e7, 21), (0.04, -1e30, 3)])
def test_stabilizer_parameters(oracle_lib, k, thr, window):
    import hmpano

    prev, nxt = moving_pair(97, 131, (-2, 1), seed=7)
    ref = oracle_lib.Stabilize(k=k, threshold=thr, window=window).run(prev, nxt)
    st = hmpano.Stabilizer(131, 97)
    out = _dev(np.zeros((97, 131), np.float32))
    st.run(_dev(prev), _dev(nxt), out, k=k, threshold=thr, window_size=window)
    _check(st, ref, out)


def test_feature_cap(oracle_lib):
    import hmpano

    prev, nxt = moving_pair(200, 300, (3, -1), seed=9)
    ref = oracle_lib.Stabilize(max_features=25).run(prev, nxt)
    assert ref["found"] > 25
    st = hmpano.Stabilizer(300, 200, max_features=25)
    out = _dev(np.zeros((200, 300), np.float32))
    st.run(_dev(prev), _dev(nxt), out)
    xy, flow, m = st.features()
    assert m.corners == ref["found"] and m.kept == 25
    assert np.array_equal(xy, ref["corners"]) and np.array_equal(flow, ref["flow"])
    assert (m.dx, m.dy) == (ref["dx"], ref["dy"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])


def test_caller_features_on_the_border(oracle_lib):
    import hmpano

    h, w = 64, 80
    prev, nxt = moving_pair(h, w, (1, 2), seed=11)
    feats = np.array([[0, 0], [w - 1, h - 1], [0, h - 1], [w - 1, 0], [1, 1], [40, 30], [40, 30], [7, 60]], np.int32)
    ref = oracle_lib.Stabilize().run(prev, nxt, features=feats)
    st = hmpano.Stabilizer(w, h, max_features=len(feats))
    p, n = _dev(prev), _dev(nxt)
    st.set_features(feats)
    st.flow(p, n)
    out = _dev(np.zeros((h, w), np.float32))
    st.warp(n, out)
    xy, flow, m = st.features()
    assert np.array_equal(xy, feats)
    assert np.array_equal(flow, ref["flow"])
    assert (m.dx, m.dy) == (ref["dx"], ref["dy"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])


def test_flat_frame_has_no_corners_and_no_motion(oracle_lib):
    import hmpano

    prev = np.full((50, 70), 3.0, np.float32)
    nxt = texture(50, 70, seed=2)
    ref = oracle_lib.Stabilize().run(prev, nxt)
    st = hmpano.Stabilizer(70, 50)
    out = _dev(np.zeros((50, 70), np.float32))
    st.run(_dev(prev), _dev(nxt), out)
    _, _, m = st.features()
    assert m.corners == 0 and (m.dx, m.dy, m.shift_x, m.shift_y) == (0.0, 0.0, 0, 0)
    assert np.array_equal(out.cpu().numpy(), nxt) and np.array_equal(ref["out"], nxt)


def test_in_place_warp_as_the_reference(oracle_lib):
    """stabilizeFrame warps d_frame in place (cudaStabilize.cu:254-266)."""
    import hmpano

    prev, nxt = moving_pair(120, 200, (-4, -2), seed=13)
    ref = oracle_lib.Stabilize().run(prev, nxt)
    st = hmpano.Stabilizer(200, 120)
    n = _dev(nxt)
    st.run(_dev(prev), n)  # out defaults to next
    _check(st, ref, n)


def test_sequence_through_one_stabilizer(oracle_lib):
    import hmpano

    h, w = 180, 256
    big = texture(h + 40, w + 40, seed=17)
    frames = [np.ascontiguousarray(big[20 - t:20 - t + h, 20 - 2 * t:20 - 2 * t + w]) for t in range(5)]
    st = hmpano.Stabilizer(w, h)
    out = _dev(np.zeros((h, w), np.float32))
    for a, b in zip(frames, frames[1:]):
        ref = oracle_lib.Stabilize().run(a, b)
        st.run(_dev(a), _dev(b), out)
        _check(st, ref, out)


def test_graph_capture_replays_identically(oracle_lib):
    import torch

    import hmpano

    h, w = 240, 320
    prev, nxt = moving_pair(h, w, (2, -2), seed=19)
    p, n = _dev(prev), _dev(nxt)
    out = _dev(np.zeros((h, w), np.float32))
    st = hmpano.Stabilizer(w, h)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        st.run(p, n, out, stream=s)  # warm-up outside capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st.run(p, n, out, stream=s)
    prev2, nxt2 = moving_pair(h, w, (-1, 3), seed=23)
    p.copy_(_dev(prev2))
    n.copy_(_dev(nxt2))
    out.zero_()
    g.replay()
    torch.cuda.synchronize()
    _check(st, oracle_lib.Stabilize().run(prev2, nxt2), out)


def test_unaligned_frames(oracle_lib):
    """Frames 4 bytes off a 16-byte boundary take the scalar flow kernel; the result is the same."""
    import torch

    import hmpano

    h, w = 90, 130
    prev, nxt = moving_pair(h, w, (2, 1), seed=31)
    ref = oracle_lib.Stabilize().run(prev, nxt)
    bufs = [torch.zeros(h * w + 1, dtype=torch.float32, device="cuda") for _ in range(3)]
    p, n, out = (b[1:].view(h, w) for b in bufs)
    p.copy_(_dev(prev))
    n.copy_(_dev(nxt))
    assert p.data_ptr() % 16 == 4
    st = hmpano.Stabilizer(w, h)
    st.run(p, n, out)
    _check(st, ref, out)
