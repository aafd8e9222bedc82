"""hmp_blend2_noalloc (the two-image pyramid blend working in the library's static scratch array),
called through the C ABI, against hmp_stitcher_process of the equivalent two-image stitcher:
identity tables, both images at (0, 0), minimize_blend off.

Both paths run the same FP32 kernels on the same values, so the tolerance is the FP32 one of the
parity tests: bit-exact. Blends of different sizes and depths (one level up to the deepest
supported, seven) run back to back, so that each one after the first reads scratch the one before
it left behind. The file is named to be collected last and
passes alone in a fresh process as well as after the other tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_stitch, make_stitcher

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as hmp_build
    import torch

    hmp_build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _frames(rng, batch, h, w, hole):
    f = rng.integers(0, 256, size=(batch, h, w, 4), dtype=np.uint8)
    f[..., 3] = 255
    y0, y1, x0, x1 = hole
    f[:, y0:y1, x0:x1, 3] = 0  # unmapped area: the blend falls back to the other image
    return f


def _seam(rng, h, w):
    xs = np.arange(w)[None, :]
    edge = (w // 2 + (w // 6) * np.sin(np.arange(h) / 17.0)).astype(np.int64)[:, None]
    seam = (xs < edge).astype(np.uint8)  # 1 = image 1 (left), 0 = image 2
    seam[rng.random((h, w)) < 0.01] ^= 1
    return seam


def _stitcher_blend(img1, img2, seam, levels, batch):
    import hmpano

    h, w = seam.shape
    mx = np.broadcast_to(np.arange(w, dtype=np.uint16)[None, :], (h, w)).copy()
    my = np.broadcast_to(np.arange(h, dtype=np.uint16)[:, None], (h, w)).copy()
    m = hmpano.ControlMasks()
    m.img1_col, m.img1_row, m.img2_col, m.img2_row = mx, my, mx, my
    m.whole_seam_mask_image = seam
    m.positions = [hmpano.SpatialTiff(0.0, 0.0), hmpano.SpatialTiff(0.0, 0.0)]
    st = make_stitcher(2, m, levels, batch, minimize=False)
    assert st.status.ok(), st.status
    return gpu_stitch(st, [img1, img2])


def _noalloc(lib, a, b, seam_dev, levels, batch, out):
    import torch
    from hmpano.pano import _image

    ia, ib, io = _image(a), _image(b), _image(out)
    stream = torch.cuda.current_stream().cuda_stream
    return lib.hmp_blend2_noalloc(C.byref(ia), C.byref(ib), C.c_void_p(seam_dev.data_ptr()), seam_dev.stride(0),
                                  levels, batch, C.byref(io), C.c_void_p(stream))


def test_noalloc_blend_matches_stitcher_twice_in_a_row():
    import torch
    from hmpano import _lib

    lib = _lib.lib()
    rng = np.random.default_rng(20261203)
    cases = [
        # (height, width, levels, batch, unmapped rectangle of image 2)
        (360, 640, 5, 1, (40, 120, 300, 420)),
        (301, 517, 4, 2, (150, 301, 0, 90)),
        (123, 200, 1, 1, (10, 60, 20, 90)),  # one level: pyr_fine alone, no coarser levels
        (360, 640, 7, 1, (200, 330, 500, 640)),  # the deepest pyramid supported (64-pixel alignment)
    ]
    prepared = []
    for h, w, levels, batch, hole in cases:
        img1 = _frames(rng, batch, h, w, (0, 0, 0, 0))
        img2 = _frames(rng, batch, h, w, hole)
        seam = _seam(rng, h, w)
        expected = _stitcher_blend(img1, img2, seam, levels, batch)
        prepared.append((img1, img2, seam, levels, batch, expected))

    dev_in = []
    for img1, img2, seam, levels, batch, _ in prepared:
        # The seam rows get a pitch above the width, as a caller's pitched buffer would.
        h, w = seam.shape
        seam_dev = torch.zeros((h, w + 13), dtype=torch.uint8, device="cuda")
        seam_dev[:, :w] = torch.from_numpy(seam).cuda()
        out = torch.full((batch, h, w, 4), 77, dtype=torch.uint8, device="cuda")
        dev_in.append((torch.from_numpy(img1).cuda(), torch.from_numpy(img2).cuda(), seam_dev, out))
    torch.cuda.synchronize()

    # Calls in a row on one stream; each reuses the scratch the one before it wrote.
    for (img1, img2, seam, levels, batch, _), (a, b, seam_dev, out) in zip(prepared, dev_in):
        s = _noalloc(lib, a, b, seam_dev, levels, batch, out)
        assert s.code == 0, s.message.decode()
    torch.cuda.synchronize()

    for (img1, img2, seam, levels, batch, expected), (_, _, _, out) in zip(prepared, dev_in):
        got = out.cpu().numpy()
        assert got.shape == expected.shape
        diff = np.abs(got.astype(np.int32) - expected.astype(np.int32))
        assert int(diff.max()) == 0, (seam.shape, levels, batch, int(diff.max()), int((diff > 0).sum()))


def test_noalloc_blend_rejects_sizes_beyond_the_static_scratch():
    import torch
    from hmpano import _lib

    lib = _lib.lib()
    # 4000 x 4000 pixels need about 340 MB of scratch; nothing is launched for a rejected size.
    h = w = 4000
    a = torch.zeros((1, h, w, 4), dtype=torch.uint8, device="cuda")
    seam = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    s = _noalloc(lib, a, a, seam, 6, 1, a)
    assert s.code == 1  # cudaErrorInvalidValue
    assert b"static maximum" in s.message and str(_lib.NOALLOC_SCRATCH_BYTES).encode() in s.message
