"""Seeded synthetic stitching workloads.

No public dataset is involved: every workload is generated from a seed. A rig is N pinhole
cameras placed on a horizontal arc and projected onto a cylindrical canvas, the way Hugin's
``nona`` exports remap tables for the reference (src/pano/controlMasks.cpp:273-326 loads them):

* remap tables are per-canvas-pixel ``uint16`` x/y source coordinates, nearest neighbour
  (``floor(x + 0.5)``), with ``65535`` in both tables where no source pixel exists;
* each table covers its camera's footprint columns over the full canvas height, placed at an
  integer canvas position (top-left of the footprint);
* the first table starts at canvas column 0 and the last one ends at the canvas width, so the
  canvas is exactly the requested size;
* seams are seeded random walks (one per adjacent overlap); two-image seams use the
  reference's inverted convention (1 = image 1, 0 = image 2) and N-image seams use labels;
* frames are RGBA uint8 (alpha 255) band-limited noise plus smooth gradients.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SENTINEL = 65535


@dataclass
class Rig:
    canvas_w: int
    canvas_h: int
    src_w: list[int]
    src_h: list[int]
    map_x: list[np.ndarray]
    map_y: list[np.ndarray]
    pos_x: list[int]
    pos_y: list[int]
    seam: np.ndarray  # uint8, canvas sized
    kind: int  # 2 = two-image stitcher, 3 = three-image, 1 = N-image
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.map_x)


def _blur(a: np.ndarray, sigma: float) -> np.ndarray:
    try:
        from scipy.ndimage import gaussian_filter

        return gaussian_filter(a, sigma=(sigma, sigma, 0), mode="reflect")
    except Exception:  # pragma: no cover - scipy is present on both machines
        r = int(3 * sigma)
        k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
        k /= k.sum()
        out = a
        for axis in (0, 1):
            out = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), axis, out)
        return out


def make_frame(width: int, height: int, seed: int, batch: int = 1) -> np.ndarray:
    """RGBA uint8 frame(s) [batch, h, w, 4]: clip(128 + 40*blur(N(0,1), 2) + 60*ramp + 20*sin)."""
    out = np.empty((batch, height, width, 4), dtype=np.uint8)
    for b in range(batch):
        rng = np.random.default_rng(seed * 1000 + b)
        noise = rng.standard_normal((height, width, 3)).astype(np.float32)
        noise = _blur(noise, 2.0)
        noise *= 1.0 / max(float(noise.std()), 1e-6)
        ys = np.linspace(-1.0, 1.0, height, dtype=np.float32)[:, None, None]
        xs = np.linspace(-1.0, 1.0, width, dtype=np.float32)[None, :, None]
        phase = rng.uniform(0, 2 * math.pi, size=3).astype(np.float32)
        ramp = (0.6 * xs + 0.4 * ys) * np.array([1.0, -0.5, 0.25], dtype=np.float32)
        wave = np.sin(2 * math.pi * (1.5 * xs + 0.7 * ys) + phase)
        v = 128.0 + 40.0 * noise + 60.0 * ramp + 20.0 * wave
        out[b, :, :, :3] = np.clip(v, 0, 255).astype(np.uint8)
        out[b, :, :, 3] = 255
    return out


def _solve_geometry(canvas_w: int, canvas_h: int, n: int, src_w: int, src_h: int, overlap: float,
                    yaw_step_deg: float | None, h_frac: float) -> tuple[float, float, float, float, float]:
    """Canvas focal fc, yaw step, horizontal FOV, source focal fs and vertical canvas scale fcv such
    that n footprints of width fc*hfov, spaced fc*step apart, span canvas_w with the requested
    pairwise overlap and each frame spans h_frac of the canvas height."""
    if yaw_step_deg is not None:
        step = math.radians(yaw_step_deg)
        if overlap <= 1.0:
            fc = canvas_w / (step * (n - 1 + 1.0 / (1.0 - overlap)))
            hfov = step / (1.0 - overlap)
        else:
            fc = (canvas_w - overlap) / (n * step)
            hfov = step + overlap / fc
    else:
        hfov = math.radians(65.0)
        ov = overlap if overlap > 1.0 else overlap * canvas_w / (n - (n - 1) * overlap)
        fc = (canvas_w + (n - 1) * ov) / (n * hfov)
        step = hfov - ov / fc
    fs = (src_w / 2.0) / math.tan(hfov / 2.0)
    fcv = h_frac * canvas_h * fs / src_h
    return fc, step, hfov, fs, fcv


def _project(canvas_w: int, canvas_h: int, fc: float, fcv: float, fs: float, src_w: int, src_h: int, yaw: float,
             roll: float) -> tuple[np.ndarray, np.ndarray]:
    """Cylindrical canvas (u, v) -> camera (yaw, roll) -> pinhole pixel, nearest neighbour. The canvas
    is an open strip: a camera only sees canvas columns within 90 degrees of its own yaw."""
    mx = np.full((canvas_h, canvas_w), SENTINEL, dtype=np.uint16)
    my = np.full((canvas_h, canvas_w), SENTINEL, dtype=np.uint16)
    cxc, cyc = canvas_w / 2.0, canvas_h / 2.0
    cxs, cys = src_w / 2.0, src_h / 2.0
    theta = (np.arange(canvas_w, dtype=np.float64) - cxc) / fc
    st, ct = np.sin(theta), np.cos(theta)
    cy_, sy_ = math.cos(yaw), math.sin(yaw)
    cr, sr = math.cos(roll), math.sin(roll)
    chunk = 256
    for v0 in range(0, canvas_h, chunk):
        v1 = min(canvas_h, v0 + chunk)
        h = ((np.arange(v0, v1, dtype=np.float64) - cyc) / fcv)[:, None]
        X, Y, Z = st[None, :], h, ct[None, :]
        # world -> camera: undo yaw about the vertical axis, then roll about the optical axis
        shape = (v1 - v0, canvas_w)
        xc = np.broadcast_to(cy_ * X - sy_ * Z, shape)
        zc = np.broadcast_to(sy_ * X + cy_ * Z, shape)
        yc = np.broadcast_to(Y, shape)
        xr = cr * xc - sr * yc
        yr = sr * xc + cr * yc
        with np.errstate(divide="ignore", invalid="ignore"):
            px = np.floor(fs * xr / zc + cxs + 0.5)
            py = np.floor(fs * yr / zc + cys + 0.5)
        front = (np.abs(theta - yaw) < math.pi / 2)[None, :]
        ok = front & (zc > 1e-6) & (px >= 0) & (px < src_w) & (py >= 0) & (py < src_h)
        bx = mx[v0:v1]
        by = my[v0:v1]
        bx[ok] = px[ok].astype(np.uint16)
        by[ok] = py[ok].astype(np.uint16)
    return mx, my


def _random_walk(rng: np.random.Generator, height: int, lo: int, hi: int) -> np.ndarray:
    lo, hi = int(lo), int(max(lo, hi))
    pos = np.empty(height, dtype=np.int64)
    x = (lo + hi) // 2
    steps = rng.integers(-1, 2, size=height)
    for y in range(height):
        x = min(max(x + int(steps[y]), lo), hi)
        pos[y] = x
    return pos


def make_rig(canvas_w: int, canvas_h: int, n: int, src_w: int, src_h: int, overlap: float, seed: int,
             kind: int | None = None, yaw_step_deg: float | None = None, roll_deg: float = 2.0, h_frac: float = 0.97,
             oob_fraction: float = 0.0) -> Rig:
    """Seeded cylindrical rig of n cameras on a canvas_w x canvas_h canvas.

    overlap: pairwise overlap, in canvas pixels if > 1, else as a fraction of a footprint width.
    kind: stitcher kind the seam is made for (2 = two-image inverted seam, else labels).
    oob_fraction: fraction of sentinel table entries replaced by out-of-range, non-sentinel
    coordinates (exercises the reference's alpha = 255 rule for such entries).
    """
    if kind is None:
        kind = 2 if n == 2 else 1
    rng = np.random.default_rng(seed)
    fc, step, hfov, fs, fcv = _solve_geometry(canvas_w, canvas_h, n, src_w, src_h, overlap, yaw_step_deg, h_frac)
    yaws = [(-(n - 1) / 2.0 + i) * step + rng.uniform(-0.002, 0.002) for i in range(n)]
    rolls = [math.radians(rng.uniform(-roll_deg, roll_deg)) for _ in range(n)]
    maps_x, maps_y, pos_x, pos_y = [], [], [], []
    col_ranges = []
    for i in range(n):
        mx, my = _project(canvas_w, canvas_h, fc, fcv, fs, src_w, src_h, yaws[i], rolls[i])
        valid_cols = np.nonzero((mx != SENTINEL).any(axis=0))[0]
        c0 = int(valid_cols[0]) if valid_cols.size else 0
        c1 = int(valid_cols[-1]) + 1 if valid_cols.size else canvas_w
        if i == 0:
            c0 = 0
        if i == n - 1:
            c1 = canvas_w
        col_ranges.append((c0, c1))
        tx = np.ascontiguousarray(mx[:, c0:c1])
        ty = np.ascontiguousarray(my[:, c0:c1])
        if oob_fraction > 0:
            sel = (tx == SENTINEL) & (rng.random(tx.shape) < oob_fraction)
            tx[sel] = src_w + 3
            ty[sel] = src_h + 3
        maps_x.append(tx)
        maps_y.append(ty)
        pos_x.append(c0)
        pos_y.append(0)
    # seams: one random walk per adjacent overlap
    seam = np.zeros((canvas_h, canvas_w), dtype=np.uint8)
    cols = np.arange(canvas_w)[None, :]
    label = np.zeros((canvas_h, canvas_w), dtype=np.int32)
    for i in range(n - 1):
        lo_edge = col_ranges[i + 1][0]
        hi_edge = col_ranges[i][1]
        if hi_edge <= lo_edge:
            mid = (lo_edge + hi_edge) // 2
            lo_edge, hi_edge = mid - 1, mid + 1
        margin = max(1, (hi_edge - lo_edge) // 6)
        walk = _random_walk(rng, canvas_h, lo_edge + margin, hi_edge - margin)
        label += (cols >= walk[:, None]).astype(np.int32)
    if kind == 2:
        seam[:] = (label == 0).astype(np.uint8)  # inverted convention: 1 = image 1
    else:
        seam[:] = label.astype(np.uint8)
    meta = {
        "hfov_deg": math.degrees(hfov),
        "yaw_step_deg": math.degrees(step),
        "fc": fc,
        "fcv": fcv,
        "fs": fs,
        "overlap_px": [col_ranges[i][1] - col_ranges[i + 1][0] for i in range(n - 1)],
    }
    return Rig(canvas_w, canvas_h, [src_w] * n, [src_h] * n, maps_x, maps_y, pos_x, pos_y, seam, kind, meta)


# Workloads named after what they are (sizes as in the reference's headline use case: two 5K
# frames onto a ~8500x3300 canvas, README.md:1-7).
WORKLOADS = {
    # two 1280x720 frames -> 2200x800 canvas, ~300 px overlap, hard seam
    "pano2_1280x720_to_2200x800": dict(canvas_w=2200, canvas_h=800, n=2, src_w=1280, src_h=720, overlap=300,
                                       yaw_step_deg=50.0),
    # two 5120x2880 frames -> 8500x3300 canvas (production)
    "pano2_5120x2880_to_8500x3300": dict(canvas_w=8500, canvas_h=3300, n=2, src_w=5120, src_h=2880, overlap=300,
                                         yaw_step_deg=60.0),
    # eight 2000x1500 frames -> 9000x2400 canvas, ~25% pairwise overlap
    "panon8_2000x1500_to_9000x2400": dict(canvas_w=9000, canvas_h=2400, n=8, src_w=2000, src_h=1500, overlap=0.25,
                                          yaw_step_deg=45.0),
    # three 2704x1520 frames -> 6000x1800 canvas
    "pano3_2704x1520_to_6000x1800": dict(canvas_w=6000, canvas_h=1800, n=3, src_w=2704, src_h=1520, overlap=0.2,
                                         yaw_step_deg=50.0),
}


def workload_rig(name: str, seed: int = 1234, kind: int | None = None, scale: float = 1.0, **kw) -> Rig:
    p = dict(WORKLOADS[name])
    p.update(kw)
    if scale != 1.0:
        for key in ("canvas_w", "canvas_h", "src_w", "src_h"):
            p[key] = max(16, int(round(p[key] * scale)))
        if p["overlap"] > 1:
            p["overlap"] = max(8, int(round(p["overlap"] * scale)))
    return make_rig(seed=seed, kind=kind, **p)


def rig_frames(rig: Rig, seed: int, batch: int = 1) -> list[np.ndarray]:
    return [make_frame(rig.src_w[i], rig.src_h[i], seed * 31 + i, batch) for i in range(rig.n)]
