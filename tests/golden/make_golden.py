"""Generate golden stitch vectors from the reference's own Python implementation.

Runs hm-cupano's ``cupano`` package (its torch CPU path, ``backend="auto"`` on CPU tensors resolves
to ``torch_impl``: cupano/ops.py:60-69) on small seeded rigs and stores inputs and outputs in
``golden.npz``. The reference imports cv2/tifffile/PIL at module load (cupano/pano.py:7,
cupano/masks.py:7-10) but only uses them for file I/O; none is installed here, so empty stand-in
modules are registered first and the ControlMasks are filled in memory (as the reference's own
tests do, tests/python/test_pytorch_pano.py:62-85).

Usage: python tests/golden/make_golden.py [--reference /path/to/hm-cupano]

One correction is applied to the port before it runs. Its workspace path builds the mask
pyramid with ``downsample_mask(..., out=buf)``, but ``_downsample_mask_torch`` returns
``out / count`` as a new tensor and leaves the un-normalised 2x2 *sum* in ``buf``
(cupano/ops.py:409-424), so levels >= 1 of the mask pyramid are 4**l times too large. The
reference's CUDA kernels divide by the count (src/cuda/cudaBlend.cu:268-296,
src/cuda/cudaBlendN.cu:19-48), and so does the port's own non-workspace path. The generator
writes the mean into ``buf``, which makes the workspace path equal to the non-workspace path
and to the CUDA semantics. Without it, two-image blends with >= 2 levels extrapolate by the
mask sum. The same holds for ``_downsample_image_torch`` with 3-channel (RGB) pixels (its
4-channel branch writes the mean into ``out``; the 3-channel branch returns ``out / count`` and
leaves the 2x2 sum in ``out``, cupano/ops.py:445-492), and the same correction is applied, as the
CUDA kernels divide by the count (src/cuda/cudaBlend.cu:46-144).

The reference tree is only needed to regenerate the fixture; the tests read ``golden.npz``.
"""
from __future__ import annotations

import argparse
import os
import sys
import types
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "hm-cupano_gb300"))

from hmpano import synth  # noqa: E402


def _install_stubs() -> None:
    cv2 = types.ModuleType("cv2")
    cv2.IMREAD_ANYDEPTH = 2
    cv2.IMREAD_GRAYSCALE = 0
    cv2.imread = lambda *a, **k: None
    cv2.imwrite = lambda *a, **k: True
    sys.modules.setdefault("cv2", cv2)
    sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    pil = types.ModuleType("PIL")
    pil.Image = types.ModuleType("PIL.Image")
    sys.modules.setdefault("PIL", pil)
    sys.modules.setdefault("PIL.Image", pil.Image)


def install_corrections(ref_ops) -> None:
    """The port's workspace downsamples leave the 2x2 sum in their output buffer (module
    docstring); write the mean there, as the CUDA kernels do."""
    sum_only = ref_ops._downsample_mask_torch

    def _downsample_mask_mean(mask, out=None):
        result = sum_only(mask, out=out)
        if out is not None:
            out.copy_(result)
            return out
        return result

    ref_ops._downsample_mask_torch = _downsample_mask_mean
    image_sum_only = ref_ops._downsample_image_torch

    def _downsample_image_mean(image, out=None):
        result = image_sum_only(image, out=out)
        if out is not None and result is not out:
            out.copy_(result)
            return out
        return result

    ref_ops._downsample_image_torch = _downsample_image_mean


def _cases():
    """(name, rig parameters, levels, minimize, batch, oob_fraction, frame seed)."""
    p2 = dict(canvas_w=480, canvas_h=40, n=2, src_w=230, src_h=36, overlap=90, yaw_step_deg=50.0)
    p2odd = dict(canvas_w=497, canvas_h=45, n=2, src_w=241, src_h=37, overlap=85, yaw_step_deg=50.0)
    pn3 = dict(canvas_w=420, canvas_h=48, n=3, src_w=160, src_h=40, overlap=0.25, yaw_step_deg=40.0)
    pn4 = dict(canvas_w=515, canvas_h=37, n=4, src_w=150, src_h=30, overlap=0.3, yaw_step_deg=35.0)
    return [
        ("pano2_l0", p2, 0, True, 1, 0.0, 11),
        ("pano2_l1", p2, 1, True, 1, 0.0, 12),
        ("pano2_l3", p2, 3, True, 1, 0.0, 13),
        ("pano2_l6_odd", p2odd, 6, True, 1, 0.0, 14),
        ("pano2_l4_full", p2, 4, False, 1, 0.0, 15),
        ("pano2_l3_oob_b2", p2odd, 3, True, 2, 0.05, 16),
        ("pano2_l0_oob_b2", p2odd, 0, True, 2, 0.05, 17),
        ("panon3_l0", pn3, 0, True, 1, 0.0, 21),
        ("panon3_l3_min", pn3, 3, True, 1, 0.0, 22),
        ("panon3_l3_full", pn3, 3, False, 1, 0.0, 23),
        ("panon4_l2_min_oob", pn4, 2, True, 1, 0.05, 24),
        ("panon4_l5_min_b2", pn4, 5, True, 2, 0.0, 25),
    ]


def _rgb_cases():
    """3-channel (RGB, no alpha) cases: the same rigs with the frames' alpha dropped."""
    p2 = dict(canvas_w=480, canvas_h=40, n=2, src_w=230, src_h=36, overlap=90, yaw_step_deg=50.0)
    p2odd = dict(canvas_w=497, canvas_h=45, n=2, src_w=241, src_h=37, overlap=85, yaw_step_deg=50.0)
    pn3 = dict(canvas_w=420, canvas_h=48, n=3, src_w=160, src_h=40, overlap=0.25, yaw_step_deg=40.0)
    pn4 = dict(canvas_w=515, canvas_h=37, n=4, src_w=150, src_h=30, overlap=0.3, yaw_step_deg=35.0)
    return [
        ("rgb_pano2_l0", p2, 0, True, 1, 0.0, 31),
        ("rgb_pano2_l3", p2, 3, True, 1, 0.0, 32),
        ("rgb_pano2_l6_odd_oob", p2odd, 6, True, 1, 0.05, 33),
        ("rgb_pano2_l4_full_b2", p2, 4, False, 2, 0.0, 34),
        ("rgb_panon3_l0", pn3, 0, True, 1, 0.0, 35),
        ("rgb_panon3_l3_min", pn3, 3, True, 1, 0.0, 36),
        ("rgb_panon4_l5_full_b2", pn4, 5, False, 2, 0.05, 37),
    ]


def _run_reference(cupano, rig, frames, levels, minimize, batch):
    import torch

    if rig.kind == 2:
        masks = cupano.ControlMasks()
        masks.img1_col, masks.img1_row = rig.map_x[0], rig.map_y[0]
        masks.img2_col, masks.img2_row = rig.map_x[1], rig.map_y[1]
        masks.whole_seam_mask_image = rig.seam
        masks.positions = [cupano.SpatialTiff(float(rig.pos_x[i]), float(rig.pos_y[i])) for i in range(2)]
        pano = cupano.CudaStitchPano(batch, levels, masks, quiet=True, minimize_blend=minimize,
                                     enable_cuda_graphs=False)
        out = pano.process(torch.from_numpy(frames[0]), torch.from_numpy(frames[1]))
    else:
        masks = cupano.ControlMasksN()
        masks.img_col = list(rig.map_x)
        masks.img_row = list(rig.map_y)
        masks.positions = [cupano.SpatialTiff(float(rig.pos_x[i]), float(rig.pos_y[i])) for i in range(rig.n)]
        masks.whole_seam_mask_indexed = rig.seam
        pano = cupano.CudaStitchPanoN(batch, levels, masks, quiet=True, minimize_blend=minimize,
                                      enable_cuda_graphs=False)
        out = pano.process([torch.from_numpy(f) for f in frames])
    return out.numpy()


def _known_answer_cases(cupano):
    """The reference's own known-answer tests (tests/python/test_pytorch_pano.py), re-expressed
    as fixtures: identity maps, constant or patterned frames."""
    import torch

    def ident(w, h):
        return (np.tile(np.arange(w, dtype=np.uint16), (h, 1)), np.tile(np.arange(h, dtype=np.uint16)[:, None], (1, w)))

    def const(w, h, rgba):
        a = np.zeros((1, h, w, 4), dtype=np.uint8)
        a[...] = np.array(rgba, dtype=np.uint8)
        return a

    def pattern(w, h, idx):
        ys, xs = np.mgrid[0:h, 0:w]
        a = np.zeros((1, h, w, 4), dtype=np.uint8)
        a[0, ..., 0] = idx * 50 + xs % 17
        a[0, ..., 1] = idx * 50 + ys % 19
        a[0, ..., 2] = idx * 50 + (xs + ys) % 23
        a[0, ..., 3] = 255
        return a

    out = []
    # hard seam selection and single-level soft seam (test_pytorch_pano.py:109-152)
    w, h, x2 = 256, 32, 128
    seam = np.zeros((h, w + x2), dtype=np.uint8)
    seam[:, :192] = 1
    mx, my = ident(w, h)
    for levels in (0, 1):
        rig = synth.Rig(w + x2, h, [w, w], [h, h], [mx, mx], [my, my], [0, x2], [0, 0], seam, 2)
        frames = [const(w, h, (10, 20, 30, 255)), const(w, h, (100, 110, 120, 255))]
        out.append((f"kat_pano2_select_l{levels}", rig, frames, levels, True, 1))
    # minimize == full (test_pytorch_pano.py:155-189)
    w, h, x2 = 384, 64, 192
    seam = np.zeros((h, w + x2), dtype=np.uint8)
    seam[:, : (w + x2) // 2] = 1
    mx, my = ident(w, h)
    for mini in (True, False):
        rig = synth.Rig(w + x2, h, [w, w], [h, h], [mx, mx], [my, my], [0, x2], [0, 0], seam, 2)
        out.append((f"kat_pano2_pattern_l4_{'min' if mini else 'full'}", rig, [pattern(w, h, 0), pattern(w, h, 1)], 4,
                    mini, 1))
    # N minimize == full (test_pytorch_pano.py:204-220)
    w = h = 64
    seam = np.zeros((h, w), dtype=np.uint8)
    seam[:, w // 2:] = 1
    mx, my = ident(w, h)
    for mini in (True, False):
        rig = synth.Rig(w, h, [w, w], [h, h], [mx, mx], [my, my], [0, 0], [0, 0], seam, 1)
        out.append((f"kat_panon2_pattern_l4_{'min' if mini else 'full'}", rig, [pattern(w, h, 0), pattern(w, h, 1)],
                    4, mini, 1))
    # N hard seam indexed selection (test_pytorch_pano.py:223-246)
    w, h = 48, 24
    seam = np.zeros((h, w), dtype=np.uint8)
    seam[:, 16:32] = 1
    seam[:, 32:] = 2
    mx, my = ident(w, h)
    rig = synth.Rig(w, h, [w] * 3, [h] * 3, [mx] * 3, [my] * 3, [0] * 3, [0] * 3, seam, 1)
    frames = [const(w, h, (10, 0, 0, 255)), const(w, h, (0, 20, 0, 255)), const(w, h, (0, 0, 30, 255))]
    out.append(("kat_panon3_select_l0", rig, frames, 0, True, 1))
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("HM_CUPANO_REFERENCE"),
                    required="HM_CUPANO_REFERENCE" not in os.environ,
                    help="the hm-cupano checkout (default: $HM_CUPANO_REFERENCE)")
    ap.add_argument("--out", default=str(HERE / "golden.npz"))
    args = ap.parse_args()
    _install_stubs()
    sys.path.insert(0, args.reference)
    import torch

    torch.set_num_threads(max(1, os.cpu_count() or 1))
    import cupano
    from cupano import ops as ref_ops
    from cupano.ops import compute_laplacian

    install_corrections(ref_ops)

    store: dict[str, np.ndarray] = {}
    names = []

    def put(name, rig, frames, levels, minimize, batch):
        canvas = _run_reference(cupano, rig, frames, levels, minimize, batch)
        pre = f"{name}/"
        store[pre + "meta"] = np.array([rig.kind, rig.n, levels, int(minimize), batch, rig.canvas_w, rig.canvas_h],
                                       dtype=np.int64)
        store[pre + "pos"] = np.array([rig.pos_x, rig.pos_y], dtype=np.int64)
        store[pre + "seam"] = rig.seam
        for i in range(rig.n):
            store[pre + f"map_x{i}"] = rig.map_x[i]
            store[pre + f"map_y{i}"] = rig.map_y[i]
            store[pre + f"frame{i}"] = frames[i]
        store[pre + "canvas"] = canvas
        names.append(name)
        print(f"{name}: canvas {canvas.shape}")

    for name, params, levels, minimize, batch, oob, fseed in _cases():
        kind = 2 if params["n"] == 2 else 1
        rig = synth.make_rig(seed=zlib.crc32(name.encode()) % 10000 + 7, kind=kind, oob_fraction=oob, **params)
        frames = [synth.make_frame(rig.src_w[i], rig.src_h[i], fseed * 10 + i, batch) for i in range(rig.n)]
        put(name, rig, frames, levels, minimize, batch)
    for name, rig, frames, levels, minimize, batch in _known_answer_cases(cupano):
        put(name, rig, frames, levels, minimize, batch)
    for name, params, levels, minimize, batch, oob, fseed in _rgb_cases():
        kind = 2 if params["n"] == 2 else 1
        rig = synth.make_rig(seed=zlib.crc32(name.encode()) % 10000 + 7, kind=kind, oob_fraction=oob, **params)
        frames = [synth.make_frame(rig.src_w[i], rig.src_h[i], fseed * 10 + i, batch)[..., :3].copy()
                  for i in range(rig.n)]
        put(name, rig, frames, levels, minimize, batch)

    # Op-level known answer: the alpha-renormalised Laplacian (test_pytorch_pano.py:192-201).
    high = torch.zeros((1, 4, 4, 4), dtype=torch.float32)
    low = torch.zeros((1, 2, 2, 4), dtype=torch.float32)
    low[:, 1, 1, :] = torch.tensor([100.0, 110.0, 120.0, 255.0])
    store["op_laplacian/high"] = high.numpy()
    store["op_laplacian/low"] = low.numpy()
    store["op_laplacian/lap"] = compute_laplacian(high, low, backend="auto").numpy()
    # Op-level: downsample / laplacian / reconstruct on seeded random RGBA with alpha holes.
    from cupano.ops import _downsample_image_torch, _reconstruct_level_torch, _downsample_mask_torch

    rng = np.random.default_rng(5)
    img = rng.uniform(0, 255, size=(1, 13, 11, 4)).astype(np.float32)
    img[..., 3] = np.where(rng.random((1, 13, 11)) < 0.3, 0.0, 255.0)
    t = torch.from_numpy(img)
    low_t = _downsample_image_torch(t)
    lap_t = compute_laplacian(t, low_t, backend="auto")
    rec_t = _reconstruct_level_torch(low_t, lap_t)
    mask = rng.uniform(0, 1, size=(13, 11, 3)).astype(np.float32)
    store["op_pyr/img"] = img
    store["op_pyr/down"] = low_t.numpy()
    store["op_pyr/lap"] = lap_t.numpy()
    store["op_pyr/rec"] = rec_t.numpy()
    store["op_pyr/mask"] = mask
    store["op_pyr/mask_down"] = _downsample_mask_torch(torch.from_numpy(mask)).numpy()
    store["names"] = np.array(names)
    np.savez_compressed(args.out, **store)
    print(f"wrote {args.out} ({Path(args.out).stat().st_size / 1024:.1f} KiB)")


if __name__ == "__main__":
    main()
