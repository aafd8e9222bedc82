"""ctypes binding of the C oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this module:
it is the checker for the CUDA path, never the thing measured or shipped. ``build()`` compiles
``hmp_oracle.c`` with gcc (no fused multiply-add, OpenMP) into ``oracle/liboracle.so``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

KIND_PANON = 1
KIND_PANO2 = 2
KIND_PANO3 = 3
FILTER_REFBOX = 0
FILTER_BINOMIAL5 = 1


def build(force: bool = False) -> Path:
    src = [HERE / "hmp_oracle.c", HERE / "hmp_oracle_body.h", HERE / "hmp_oracle.h", HERE / "hmp_stabilize_oracle.c"]
    if LIB_PATH.exists() and not force and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
           "-o", str(LIB_PATH) + ".tmp", str(HERE / "hmp_oracle.c"), str(HERE / "hmp_stabilize_oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(str(LIB_PATH) + ".tmp", LIB_PATH)
    return LIB_PATH


class _Config(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("n_images", C.c_int),
        ("num_levels", C.c_int),
        ("batch", C.c_int),
        ("minimize_blend", C.c_int),
        ("fused3", C.c_int),
        ("filter", C.c_int),
        ("map_x", C.POINTER(C.POINTER(C.c_uint16))),
        ("map_y", C.POINTER(C.POINTER(C.c_uint16))),
        ("map_w", C.POINTER(C.c_int)),
        ("map_h", C.POINTER(C.c_int)),
        ("pos_x", C.POINTER(C.c_int)),
        ("pos_y", C.POINTER(C.c_int)),
        ("seam", C.POINTER(C.c_uint8)),
        ("seam_w", C.c_int),
        ("seam_h", C.c_int),
        ("channels", C.c_int),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        L.hmpo_canvas_size.argtypes = [P(_Config), P(C.c_int), P(C.c_int)]
        L.hmpo_blend_geometry.argtypes = [P(_Config), P(C.c_int)]
        for name in ("hmpo_stitch_f32", "hmpo_stitch_f64"):
            getattr(L, name).argtypes = [P(_Config), P(P(C.c_uint8)), P(C.c_int), P(C.c_int), P(C.c_uint8)]
        L.hmpo_stitch_f64_unpacked.argtypes = [P(_Config), P(P(C.c_uint8)), P(C.c_int), P(C.c_int), P(C.c_double)]
        L.hmpo_downsample_rgba_f32.argtypes = [P(C.c_float), C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_laplacian_rgba_f32.argtypes = [P(C.c_float), C.c_int, C.c_int, P(C.c_float), P(C.c_float)]
        L.hmpo_reconstruct_rgba_f32.argtypes = [P(C.c_float), P(C.c_float), C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_blend_two_f32.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float), C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_downsample_mask_f32.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_blend_nway_f32.argtypes = [P(P(C.c_float)), C.c_int, P(C.c_float), C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_laplacian_blend_ch_f32.argtypes = [P(P(C.c_float)), C.c_int, P(C.c_float), C.c_int, C.c_int, C.c_int,
                                                  C.c_int, C.c_int, C.c_int, P(C.c_float)]
        L.hmpo_laplacian_blend_ch_f32.restype = C.c_int
        L.hmpo_stab_harris.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_float, P(C.c_float), P(C.c_float),
                                       P(C.c_float)]
        L.hmpo_stab_corners.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_float, P(C.c_int), C.c_int]
        L.hmpo_stab_corners.restype = C.c_int
        L.hmpo_stab_flow.argtypes = [P(C.c_float), P(C.c_float), P(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int,
                                     P(C.c_float)]
        L.hmpo_stab_mean.argtypes = [P(C.c_float), C.c_int, P(C.c_float), P(C.c_float)]
        L.hmpo_stab_warp.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_float, C.c_float, P(C.c_float)]
        L.hmpo_set_threads.argtypes = [C.c_int]
        L.hmpo_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


class Stitch:
    """Oracle stitch for one rig description (numpy arrays, kept alive by this object)."""

    def __init__(self, kind: int, map_x, map_y, pos_x, pos_y, seam: np.ndarray, num_levels: int, batch: int = 1,
                 minimize_blend: bool = True, fused3: bool = True, filter: int = FILTER_REFBOX):
        n = len(map_x)
        self.n = n
        self._mx = [np.ascontiguousarray(m, dtype=np.uint16) for m in map_x]
        self._my = [np.ascontiguousarray(m, dtype=np.uint16) for m in map_y]
        self._seam = np.ascontiguousarray(seam, dtype=np.uint8)
        self._mxp = (C.POINTER(C.c_uint16) * n)(*[_ptr(m, C.c_uint16) for m in self._mx])
        self._myp = (C.POINTER(C.c_uint16) * n)(*[_ptr(m, C.c_uint16) for m in self._my])
        self._mw = (C.c_int * n)(*[m.shape[1] for m in self._mx])
        self._mh = (C.c_int * n)(*[m.shape[0] for m in self._mx])
        self._px = (C.c_int * n)(*[int(v) for v in pos_x])
        self._py = (C.c_int * n)(*[int(v) for v in pos_y])
        self.cfg = _Config(kind, n, num_levels, batch, int(minimize_blend), int(fused3), filter, self._mxp, self._myp,
                           self._mw, self._mh, self._px, self._py, _ptr(self._seam, C.c_uint8), self._seam.shape[1],
                           self._seam.shape[0])
        self.batch = batch
        w, h = C.c_int(), C.c_int()
        rc = lib().hmpo_canvas_size(C.byref(self.cfg), C.byref(w), C.byref(h))
        if rc != 0:
            raise ValueError(f"oracle: invalid configuration ({rc})")
        self.canvas_w, self.canvas_h = w.value, h.value

    @classmethod
    def from_rig(cls, rig, num_levels: int, batch: int = 1, minimize_blend: bool = True, **kw) -> "Stitch":
        return cls(rig.kind, rig.map_x, rig.map_y, rig.pos_x, rig.pos_y, rig.seam, num_levels, batch,
                   minimize_blend, **kw)

    def geometry(self) -> dict:
        out = (C.c_int * 9)()
        rc = lib().hmpo_blend_geometry(C.byref(self.cfg), out)
        if rc != 0:
            raise ValueError(f"oracle: geometry failed ({rc})")
        v = list(out)
        return {"blend": tuple(v[0:4]), "write": tuple(v[4:8]), "levels": v[8]}

    def _inputs(self, frames):
        """Frames [batch, h, w, c] uint8 with c = 4 (RGBA) or 3 (RGB); sets the config's channels."""
        fr = [np.ascontiguousarray(f, dtype=np.uint8) for f in frames]
        ch = fr[0].shape[-1] if fr and fr[0].ndim == 4 else 0
        for f in fr:
            if f.ndim != 4 or f.shape[0] != self.batch or f.shape[3] != ch or ch not in (3, 4):
                raise ValueError("frames must be [batch, h, w, 4 or 3] uint8 with one channel count")
        self.cfg.channels = ch
        self.channels = ch
        ptrs = (C.POINTER(C.c_uint8) * self.n)(*[_ptr(f, C.c_uint8) for f in fr])
        ws = (C.c_int * self.n)(*[f.shape[2] for f in fr])
        hs = (C.c_int * self.n)(*[f.shape[1] for f in fr])
        return fr, ptrs, ws, hs

    def run(self, frames, precision: str = "f32") -> np.ndarray:
        fr, ptrs, ws, hs = self._inputs(frames)
        out = np.zeros((self.batch, self.canvas_h, self.canvas_w, self.channels), dtype=np.uint8)
        fn = lib().hmpo_stitch_f32 if precision == "f32" else lib().hmpo_stitch_f64
        rc = fn(C.byref(self.cfg), ptrs, ws, hs, _ptr(out, C.c_uint8))
        if rc != 0:
            raise RuntimeError(f"oracle stitch failed ({rc})")
        return out

    def run_unpacked_f64(self, frames) -> np.ndarray:
        """Pre-pack FP64 blend result of the write ROI, [batch, wh, ww, 4]."""
        g = self.geometry()
        _, _, ww, wh = g["write"]
        fr, ptrs, ws, hs = self._inputs(frames)
        out = np.zeros((self.batch, wh, ww, 4), dtype=np.float64)
        rc = lib().hmpo_stitch_f64_unpacked(C.byref(self.cfg), ptrs, ws, hs, _ptr(out, C.c_double))
        if rc != 0:
            raise RuntimeError(f"oracle stitch failed ({rc})")
        return out


def set_threads(n: int) -> None:
    lib().hmpo_set_threads(int(n))


def get_threads() -> int:
    return int(lib().hmpo_get_threads())


def downsample_rgba(img: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.float32)
    h, w = img.shape[-3], img.shape[-2]
    out = np.zeros(((h + 1) // 2, (w + 1) // 2, 4), dtype=np.float32)
    lib().hmpo_downsample_rgba_f32(_ptr(img, C.c_float), w, h, _ptr(out, C.c_float))
    return out


def laplacian_rgba(high: np.ndarray, low: np.ndarray) -> np.ndarray:
    high = np.ascontiguousarray(high, dtype=np.float32)
    low = np.ascontiguousarray(low, dtype=np.float32)
    h, w = high.shape[-3], high.shape[-2]
    out = np.zeros((h, w, 4), dtype=np.float32)
    lib().hmpo_laplacian_rgba_f32(_ptr(high, C.c_float), w, h, _ptr(low, C.c_float), _ptr(out, C.c_float))
    return out


def reconstruct_rgba(low: np.ndarray, lap: np.ndarray) -> np.ndarray:
    low = np.ascontiguousarray(low, dtype=np.float32)
    lap = np.ascontiguousarray(lap, dtype=np.float32)
    h, w = lap.shape[-3], lap.shape[-2]
    out = np.zeros((h, w, 4), dtype=np.float32)
    lib().hmpo_reconstruct_rgba_f32(_ptr(low, C.c_float), _ptr(lap, C.c_float), w, h, _ptr(out, C.c_float))
    return out


def blend_two_rgba(l1: np.ndarray, l2: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """One level of the two-image blend; mask [h, w] (or [h, w, 1]) is the weight of image 1."""
    l1 = np.ascontiguousarray(l1, dtype=np.float32)
    l2 = np.ascontiguousarray(l2, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    h, w = l1.shape[-3], l1.shape[-2]
    out = np.zeros((h, w, 4), dtype=np.float32)
    lib().hmpo_blend_two_f32(_ptr(l1, C.c_float), _ptr(l2, C.c_float), _ptr(mask, C.c_float), w, h,
                             _ptr(out, C.c_float))
    return out


def blend_nway_rgba(laps, mask: np.ndarray) -> np.ndarray:
    """One level of the N-way blend (cudaBlendN.cu:199-288): laps n x [h, w, 4], mask [h, w, n]."""
    laps = [np.ascontiguousarray(a, dtype=np.float32) for a in laps]
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    h, w = laps[0].shape[-3], laps[0].shape[-2]
    ptrs = (C.POINTER(C.c_float) * len(laps))(*[_ptr(a, C.c_float) for a in laps])
    out = np.zeros((h, w, 4), dtype=np.float32)
    lib().hmpo_blend_nway_f32(ptrs, len(laps), _ptr(mask, C.c_float), w, h, _ptr(out, C.c_float))
    return out


RULE_NWAY, RULE_TWO, RULE_THREE = 1, 2, 3


def laplacian_blend(images, mask: np.ndarray, levels: int, rule: int) -> np.ndarray:
    """The whole Laplacian blend of full float buffers (cudaBlend.cu:847-1049, cudaBlend3.cu:881-1206,
    cudaBlendN.cu:649-828): images n x [h, w, C] (C = 3 or 4), mask [h, w, k] (k = 1 for the
    two-image rule, else one weight per image); returns [h, w, C]."""
    h, w, ch = np.shape(images[0])
    if ch not in (3, 4):
        raise ValueError("images must have 3 or 4 channels")
    # The oracle's float buffers hold 4 values per pixel in both modes (the 3-channel mode
    # ignores the fourth).
    padded = []
    for a in images:
        b = np.zeros((h, w, 4), dtype=np.float32)
        b[..., :ch] = a
        padded.append(b)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    k = mask.shape[-1] if mask.ndim == 3 else 1
    ptrs = (C.POINTER(C.c_float) * len(padded))(*[_ptr(a, C.c_float) for a in padded])
    out = np.zeros((h, w, 4), dtype=np.float32)
    rc = lib().hmpo_laplacian_blend_ch_f32(ptrs, len(padded), _ptr(mask, C.c_float), k, w, h, int(levels), int(rule),
                                           ch, _ptr(out, C.c_float))
    if rc != 0:
        raise ValueError(f"laplacian_blend: oracle error {rc}")
    return out[..., :ch]


def downsample_mask(mask: np.ndarray) -> np.ndarray:
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    h, w, k = mask.shape
    out = np.zeros(((h + 1) // 2, (w + 1) // 2, k), dtype=np.float32)
    lib().hmpo_downsample_mask_f32(_ptr(mask, C.c_float), w, h, k, _ptr(out, C.c_float))
    return out


def load_golden_case(npz, name: str):
    """Unpack one golden stitch case into (kind, levels, minimize, batch, maps..., frames, canvas)."""
    meta = npz[f"{name}/meta"]
    kind, n, levels, minimize, batch = (int(v) for v in meta[:5])
    pos = npz[f"{name}/pos"]
    case = {
        "kind": kind,
        "n": n,
        "levels": levels,
        "minimize": bool(minimize),
        "batch": batch,
        "pos_x": [int(v) for v in pos[0]],
        "pos_y": [int(v) for v in pos[1]],
        "seam": npz[f"{name}/seam"],
        "map_x": [npz[f"{name}/map_x{i}"] for i in range(n)],
        "map_y": [npz[f"{name}/map_y{i}"] for i in range(n)],
        "frames": [npz[f"{name}/frame{i}"] for i in range(n)],
        "canvas": npz[f"{name}/canvas"],
    }
    return case


class Stabilize:
    """Frame stabiliser of src/cuda/cudaStabilize.cu on the CPU: Harris corners of `prev`, their
    Lucas-Kanade flow into `next`, the mean flow, and `next` translated by its rounding as the
    reference's warp does it (output (x, y) = next(x - shift_x, y - shift_y), zero outside)."""

    def __init__(self, k: float = 0.04, threshold: float = 1e6, window: int = 15, max_features: int = 0):
        self.k, self.threshold, self.window = float(k), float(threshold), int(window)
        self.max_features = int(max_features)  # 0: no limit; else only the first ones are tracked

    def run(self, prev: np.ndarray, nxt: np.ndarray, features=None) -> dict:
        """features: an (n, 2) list of (x, y) to track instead of prev's corners."""
        L = lib()
        prev = np.ascontiguousarray(prev, dtype=np.float32)
        nxt = np.ascontiguousarray(nxt, dtype=np.float32)
        h, w = prev.shape
        gx, gy, resp = (np.zeros((h, w), np.float32) for _ in range(3))
        L.hmpo_stab_harris(_ptr(prev, C.c_float), w, h, self.k, _ptr(gx, C.c_float), _ptr(gy, C.c_float),
                           _ptr(resp, C.c_float))
        found = L.hmpo_stab_corners(_ptr(resp, C.c_float), w, h, self.threshold, None, 0)
        xy = np.zeros((max(found, 1), 2), np.int32)
        L.hmpo_stab_corners(_ptr(resp, C.c_float), w, h, self.threshold, _ptr(xy, C.c_int), found)
        n = min(found, self.max_features) if self.max_features else found
        if features is not None:
            xy = np.ascontiguousarray(features, dtype=np.int32).reshape(-1, 2)
            found = n = len(xy)
            xy = xy if n else np.zeros((1, 2), np.int32)
        flow = np.zeros((max(n, 1), 2), np.float32)
        L.hmpo_stab_flow(_ptr(prev, C.c_float), _ptr(nxt, C.c_float), _ptr(xy, C.c_int), n, w, h, self.window,
                         _ptr(flow, C.c_float))
        dx, dy = C.c_float(), C.c_float()
        L.hmpo_stab_mean(_ptr(flow, C.c_float), n, C.byref(dx), C.byref(dy))
        out = np.zeros((h, w), np.float32)
        L.hmpo_stab_warp(_ptr(nxt, C.c_float), w, h, dx.value, dy.value, _ptr(out, C.c_float))
        return {"response": resp, "found": found, "corners": xy[:n], "flow": flow[:n], "dx": dx.value, "dy": dy.value,
                "out": out}
