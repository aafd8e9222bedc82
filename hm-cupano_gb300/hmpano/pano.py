"""Python mirror of the reference's stitcher API over the C ABI.

Same class names, constructor arguments, ``process`` signatures and error behaviour as the
reference's ``cupano`` package (cupano/pano.py:127-911, cupano/masks.py) and its C++ classes
(src/pano/cudaPano.h, cudaPano3.h, cudaPanoN.h):

* ``ControlMasks`` / ``ControlMasks3`` / ``ControlMasksN`` hold the already-loaded remap tables,
  positions and seam (two-image seams in the reference's inverted form, 1 = image 1);
* a stitcher whose masks are invalid keeps an error ``status`` instead of raising at
  construction, and ``process`` raises ``CudaStatusError`` while the status is not ok;
* ``process`` takes RGBA uint8 CUDA tensors ``[B, H, W, 4]`` (or ``[H, W, 4]``) and returns the
  canvas tensor (allocated when not given).

Every stitch runs in libhmpano.so's sm_103a kernels; torch only supplies device memory and the
current stream.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import Config, Image, Remap, Status, StitcherInfo

UNMAPPED_POSITION_VALUE = np.uint16(65535)


@dataclass
class SpatialTiff:
    xpos: float
    ypos: float


@dataclass
class Rect:
    """Integer rectangle of the reference's geometry module (cupano/geometry.py), exported for
    code written against it."""

    x: int = 0
    y: int = 0
    width: int = 0
    height: int = 0

    @property
    def empty(self) -> bool:
        return self.width <= 0 or self.height <= 0

    @property
    def right(self) -> int:
        return self.x + self.width

    @property
    def bottom(self) -> int:
        return self.y + self.height

    def intersect(self, other: "Rect") -> "Rect":
        x0, y0 = max(self.x, other.x), max(self.y, other.y)
        w, h = min(self.right, other.right) - x0, min(self.bottom, other.bottom) - y0
        return Rect(x0, y0, max(0, w), max(0, h))


@dataclass
class CanvasInfo:
    """Canvas size and the tables' integer positions on it (cupano/geometry.py)."""

    width: int
    height: int
    positions: list = field(default_factory=list)


@dataclass(frozen=True)
class CudaStatus:
    code: int = 0
    message: str = ""

    def ok(self) -> bool:
        return self.code == 0


class CudaStatusError(RuntimeError):
    def __init__(self, status: CudaStatus):
        self.status = status
        super().__init__(status.message or f"CudaStatus(code={status.code})")


def _status(s: Status) -> CudaStatus:
    return CudaStatus(int(s.code), s.message.decode(errors="replace"))


def _normalize_positions(positions: Sequence[SpatialTiff]) -> list[tuple[int, int]]:
    return [(int(p.xpos), int(p.ypos)) for p in positions]


class Batch:
    """A batched job through hmp_batch_*: process() calls of several stitchers, captured once into
    a CUDA graph (calls under one stream index in order, indices concurrently) and replayed with one
    launch. Inputs and canvases are fixed at add(); refill the inputs between launches."""

    def __init__(self):
        self._h = C.c_void_p()
        s = _status(_lib.lib().hmp_batch_create(C.byref(self._h)))
        if not s.ok():
            raise CudaStatusError(s)
        self._keep = []

    def add(self, stitcher, inputs: Sequence, canvas, stream_index: int = 0) -> None:
        batched = [_ensure_batched(t) for t in inputs]
        canvas = _ensure_batched(canvas)
        imgs = (Image * len(batched))(*[_image(t) for t in batched])
        cv = _image(canvas)
        handle = stitcher._handle_for(*_pixel_type(batched[0]))
        self._keep += [batched, canvas, imgs, cv, stitcher]
        s = _status(_lib.lib().hmp_batch_add(self._h, handle, imgs, len(batched), C.byref(cv), int(stream_index)))
        if not s.ok():
            raise CudaStatusError(s)

    def _stream(self, stream):
        import torch

        if stream is None:
            return torch.cuda.current_stream().cuda_stream
        return stream.cuda_stream if hasattr(stream, "cuda_stream") else stream

    def capture(self, stream=None) -> None:
        s = _status(_lib.lib().hmp_batch_capture(self._h, C.c_void_p(self._stream(stream))))
        if not s.ok():
            raise CudaStatusError(s)

    def launch(self, stream=None) -> None:
        s = _status(_lib.lib().hmp_batch_launch(self._h, C.c_void_p(self._stream(stream))))
        if not s.ok():
            raise CudaStatusError(s)

    def close(self) -> None:
        if self._h:
            _lib.lib().hmp_batch_destroy(self._h)
            self._h = C.c_void_p()
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_control_dir(directory, kind: int, n_images: int = 0) -> dict:
    """Read a control directory through hmp_control_dir_load (src/pano/controlMasks.cpp:133-326 and
    its three- and N-image forms): {"map_x": [...], "map_y": [...], "positions": [SpatialTiff],
    "seam": array}, the seam processed for `kind`. Raises CudaStatusError on failure."""
    L = _lib.lib()
    out = C.POINTER(_lib.ControlDir)()
    s = _status(L.hmp_control_dir_load(str(directory).encode(), kind, n_images, C.byref(out)))
    if not s.ok():
        raise CudaStatusError(s)
    try:
        d = out.contents

        def arr(ptr, h, w, dtype):
            return np.ctypeslib.as_array(ptr, shape=(h, w)).astype(dtype, copy=True)

        n = d.n
        return {
            "map_x": [arr(d.map_x[i], d.map_height[i], d.map_width[i], np.uint16) for i in range(n)],
            "map_y": [arr(d.map_y[i], d.map_height[i], d.map_width[i], np.uint16) for i in range(n)],
            "positions": [SpatialTiff(float(d.xpos[i]), float(d.ypos[i])) for i in range(n)],
            "seam": arr(d.seam, d.seam_height, d.seam_width, np.uint8),
        }
    finally:
        L.hmp_control_dir_free(out)


def read_seam_png(path) -> tuple[np.ndarray, bool]:
    """Decode a seam PNG: (palette indices or grayscale [h, w] uint8, whether it was 8-bit paletted)."""
    L = _lib.lib()
    w, h, pal = C.c_int(), C.c_int(), C.c_int()
    s = _status(L.hmp_read_seam_png(str(path).encode(), C.byref(w), C.byref(h), C.byref(pal), None, 0))
    if not s.ok():
        raise CudaStatusError(s)
    out = np.empty((h.value, w.value), np.uint8)
    s = _status(L.hmp_read_seam_png(str(path).encode(), C.byref(w), C.byref(h), C.byref(pal),
                                    out.ctypes.data_as(C.c_void_p), out.size))
    if not s.ok():
        raise CudaStatusError(s)
    return out, bool(pal.value)


def read_tiff_u16(path) -> np.ndarray:
    """Decode a single-channel 16-bit TIFF (a coordinate table)."""
    L = _lib.lib()
    w, h = C.c_int(), C.c_int()
    s = _status(L.hmp_read_tiff_u16(str(path).encode(), C.byref(w), C.byref(h), None, 0))
    if not s.ok():
        raise CudaStatusError(s)
    out = np.empty((h.value, w.value), np.uint16)
    s = _status(L.hmp_read_tiff_u16(str(path).encode(), C.byref(w), C.byref(h), out.ctypes.data_as(C.c_void_p),
                                    out.size))
    if not s.ok():
        raise CudaStatusError(s)
    return out


def _is_dir_arg(v) -> bool:
    return isinstance(v, (str, os.PathLike))


@dataclass
class ControlMasks:
    """Two-image control data (src/pano/controlMasks.h:30-66). ``ControlMasks(game_dir)`` loads a
    control directory, as the reference's constructor does (cupano/masks.py:82-90); the fields can
    also be given directly."""

    img1_col: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img1_row: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img2_col: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img2_row: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    whole_seam_mask_image: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint8))
    positions: list = field(default_factory=list)

    def __post_init__(self):
        if _is_dir_arg(self.img1_col):
            game_dir, self.img1_col = self.img1_col, np.empty((0, 0), np.uint16)
            self.load(game_dir)

    def is_valid(self) -> bool:
        return bool(self.img1_col.size and self.img1_row.size and self.img2_col.size and self.img2_row.size
                    and self.whole_seam_mask_image.size and len(self.positions) == 2)

    def canvas_width(self) -> int:
        return int(max(self.positions[0].xpos + self.img1_col.shape[1], self.positions[1].xpos + self.img2_col.shape[1]))

    def canvas_height(self) -> int:
        return int(max(self.positions[0].ypos + self.img1_col.shape[0], self.positions[1].ypos + self.img2_col.shape[0]))

    def _tables(self):
        return [self.img1_col, self.img2_col], [self.img1_row, self.img2_row], self.whole_seam_mask_image

    def load(self, game_dir) -> bool:
        """Read mapping_000{0,1}{,_x,_y}.tif and seam_file.png (src/pano/controlMasks.cpp:265-326); the
        seam is inverted (smallest value -> 1 = image 1). False if anything is missing or invalid."""
        try:
            d = load_control_dir(game_dir, _lib.KIND_PANO2)
        except CudaStatusError:
            return False
        self.img1_col, self.img2_col = d["map_x"]
        self.img1_row, self.img2_row = d["map_y"]
        self.whole_seam_mask_image = d["seam"]
        self.positions = d["positions"]
        return self.is_valid()

    @classmethod
    def from_directory(cls, game_dir) -> "ControlMasks":
        m = cls()
        m.load(game_dir)
        return m


@dataclass
class ControlMasks3:
    """Three-image control data (src/pano/controlMasks3.h); the seam holds labels 0, 1, 2.
    ``ControlMasks3(game_dir)`` loads a control directory, like the C++ constructor."""

    img0_col: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img0_row: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img1_col: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img1_row: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img2_col: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    img2_row: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint16))
    whole_seam_mask_image: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint8))
    positions: list = field(default_factory=list)

    def __post_init__(self):
        if _is_dir_arg(self.img0_col):
            game_dir, self.img0_col = self.img0_col, np.empty((0, 0), np.uint16)
            self.load(game_dir)

    def is_valid(self) -> bool:
        return bool(all(a.size for a in (self.img0_col, self.img0_row, self.img1_col, self.img1_row, self.img2_col,
                                          self.img2_row, self.whole_seam_mask_image)) and len(self.positions) == 3)

    def _tables(self):
        return ([self.img0_col, self.img1_col, self.img2_col], [self.img0_row, self.img1_row, self.img2_row],
                self.whole_seam_mask_image)

    def load(self, game_dir) -> bool:
        """Read mapping_000{0,1,2}{,_x,_y}.tif and seam_file.png (src/pano/controlMasks3.cpp:219-300); the
        seam must be 8-bit paletted with labels 0, 1, 2."""
        try:
            d = load_control_dir(game_dir, _lib.KIND_PANO3)
        except CudaStatusError:
            return False
        self.img0_col, self.img1_col, self.img2_col = d["map_x"]
        self.img0_row, self.img1_row, self.img2_row = d["map_y"]
        self.whole_seam_mask_image = d["seam"]
        self.positions = d["positions"]
        return self.is_valid()

    @classmethod
    def from_directory(cls, game_dir) -> "ControlMasks3":
        m = cls()
        m.load(game_dir)
        return m


@dataclass
class ControlMasksN:
    """N-image control data (src/pano/controlMasksN.h); the seam holds labels 0..N-1.
    ``ControlMasksN(directory, n_images)`` loads a control directory, as the reference's
    constructor does when both are given (cupano/masks.py:133-139)."""

    img_col: list = field(default_factory=list)
    img_row: list = field(default_factory=list)
    whole_seam_mask_indexed: np.ndarray = field(default_factory=lambda: np.empty((0, 0), np.uint8))
    positions: list = field(default_factory=list)

    def __post_init__(self):
        if _is_dir_arg(self.img_col):
            directory, n_images = self.img_col, self.img_row
            self.img_col, self.img_row = [], []
            if isinstance(n_images, int):
                self.load(directory, n_images)

    def is_valid(self) -> bool:
        return bool(self.img_col and len(self.img_col) == len(self.img_row) and len(self.positions) == len(self.img_col)
                    and self.whole_seam_mask_indexed.size > 0)

    def canvas_width(self) -> int:
        return int(max(p.xpos + m.shape[1] for p, m in zip(self.positions, self.img_col)))

    def canvas_height(self) -> int:
        return int(max(p.ypos + m.shape[0] for p, m in zip(self.positions, self.img_row)))

    @staticmethod
    def split_to_channels(indexed: np.ndarray, n_images: int) -> np.ndarray:
        return np.stack([(indexed == i).astype(np.uint8) for i in range(n_images)], axis=-1)

    def _tables(self):
        return list(self.img_col), list(self.img_row), self.whole_seam_mask_indexed

    def load(self, directory, n_images: int) -> bool:
        """Read mapping_%04d{,_x,_y}.tif for n_images images and seam_file.png
        (src/pano/controlMasksN.cpp:126-193); seam values are remapped to 0..n_images-1 and must
        number exactly n_images."""
        try:
            d = load_control_dir(directory, _lib.KIND_PANON, n_images)
        except CudaStatusError:
            return False
        self.img_col, self.img_row = d["map_x"], d["map_y"]
        self.whole_seam_mask_indexed = d["seam"]
        self.positions = d["positions"]
        return self.is_valid()

    @classmethod
    def from_directory(cls, directory, n_images: int) -> "ControlMasksN":
        m = cls()
        m.load(directory, n_images)
        return m


_STORAGE = {"f32": _lib.STORAGE_F32, "fp32": _lib.STORAGE_F32, "f16": _lib.STORAGE_F16, "fp16": _lib.STORAGE_F16}
_FILTER = {"refbox": _lib.FILTER_REFBOX, "box": _lib.FILTER_REFBOX, "binomial5": _lib.FILTER_BINOMIAL5}


def build_config(kind: int, control_masks, num_levels: int, batch_size: int, minimize_blend: bool = True,
                 fused: bool = True, storage: str = "f32", filter: str = "refbox", channels: int = 4,
                 float_pixels: bool = False):
    """Marshal control masks into an hmp_config; returns (config, keep-alive list)."""
    cols, rows, seam = control_masks._tables()
    positions = _normalize_positions(control_masks.positions)
    n = len(cols)
    keep = []
    remaps = (Remap * n)()
    for i in range(n):
        mx = np.ascontiguousarray(cols[i], dtype=np.uint16)
        my = np.ascontiguousarray(rows[i], dtype=np.uint16)
        if mx.shape != my.shape:
            raise ValueError(f"remap x/y tables of image {i} differ in shape")
        keep += [mx, my]
        remaps[i] = Remap(mx.ctypes.data_as(C.POINTER(C.c_uint16)), my.ctypes.data_as(C.POINTER(C.c_uint16)),
                          int(mx.shape[1]), int(mx.shape[0]), positions[i][0], positions[i][1])
    seam_u8 = np.ascontiguousarray(seam, dtype=np.uint8)
    keep += [seam_u8, remaps]
    cfg = Config(kind, n, int(num_levels), int(batch_size), int(channels), int(bool(minimize_blend)), int(bool(fused)),
                 _STORAGE[storage.lower()], _FILTER[filter.lower()], remaps,
                 seam_u8.ctypes.data_as(C.POINTER(C.c_uint8)), int(seam_u8.shape[1]) if seam_u8.ndim == 2 else 0,
                 int(seam_u8.shape[0]) if seam_u8.ndim == 2 else 0,
                 _lib.PIXEL_F32 if float_pixels else _lib.PIXEL_U8)
    return cfg, keep


def _ensure_batched(t):
    if t.dim() == 3:
        return t.unsqueeze(0)
    if t.dim() != 4:
        raise ValueError(f"Expected HWC or BHWC tensor, got shape {tuple(t.shape)}")
    return t


def _pixel_type(t) -> tuple[int, bool]:
    """(channels, float samples) of a [.., H, W, C] tensor: uint8 or float32, 3 or 4 channels."""
    import torch

    if t.shape[-1] not in (3, 4) or t.dtype not in (torch.uint8, torch.float32):
        raise ValueError("images must be uint8 or float32 tensors with 3 or 4 channels [B, H, W, C]")
    return int(t.shape[-1]), t.dtype == torch.float32


def _image(t) -> Image:
    """hmp_image over a [B, H, W, C] CUDA tensor (C = 4 or 3; uint8 or float32) with dense pixels
    and frames (the row pitch may exceed the row). The stride of a dimension of size 1 is not
    used (numpy's `a[None]` gives such an axis stride 0)."""
    ch, _ = _pixel_type(t)
    if not t.is_cuda:
        raise ValueError("images must live on a CUDA device")
    B, H, W, _ = t.shape
    pitch = t.stride(1) if H > 1 else W * ch
    if (t.stride(3) != 1 or (W > 1 and t.stride(2) != ch) or pitch < W * ch
            or (B > 1 and t.stride(0) != pitch * H)):
        raise ValueError("images need dense pixels, rows and frames (row pitch may exceed the row)")
    return Image(C.c_void_p(t.data_ptr()), int(W), int(H), int(pitch) * t.element_size())


class _Stitcher:
    _kind = 0

    def __init__(self, control_masks, num_levels: int, batch_size: int, quiet: bool, minimize_blend: bool,
                 fused: bool, storage: str, filter: str):
        self._handle = C.c_void_p()
        self._status = CudaStatus()
        self._batch = int(batch_size)
        # Stitchers for other pixel types (uchar3, float4, float3), made on first use: the
        # reference's stitchers take their pixel type from the tensors they are given.
        self._others: dict = {}
        self._args = (control_masks, num_levels, batch_size, minimize_blend, fused, storage, filter)
        if not control_masks.is_valid():
            self._status = CudaStatus(301, "Stitching masks were not able to be loaded")
            return
        cfg, keep = build_config(self._kind, control_masks, num_levels, batch_size, minimize_blend, fused, storage,
                                 filter)
        s = _lib.lib().hmp_stitcher_create(C.byref(cfg), C.byref(self._handle))
        del keep
        self._status = _status(s)
        if not quiet and self._status.ok():
            print(f"Stitched canvas size: {self.canvas_width()} x {self.canvas_height()}")

    def __del__(self):
        for h in [getattr(self, "_handle", None), *getattr(self, "_others", {}).values()]:
            if h:
                try:
                    _lib.lib().hmp_stitcher_destroy(h)
                except Exception:
                    pass
        self._handle = C.c_void_p()
        self._others = {}

    def _handle_for(self, channels: int, float_pixels: bool):
        if (channels, float_pixels) == (4, False):
            return self._handle
        h = self._others.get((channels, float_pixels))
        if h is None:
            masks, levels, batch, minimize, fused, storage, filt = self._args
            cfg, keep = build_config(self._kind, masks, levels, batch, minimize, fused, storage, filt, channels,
                                     float_pixels)
            h = C.c_void_p()
            st = _status(_lib.lib().hmp_stitcher_create(C.byref(cfg), C.byref(h)))
            del keep
            if not st.ok():
                if h:
                    _lib.lib().hmp_stitcher_destroy(h)
                raise CudaStatusError(st)
            self._others[(channels, float_pixels)] = h
        return h

    @property
    def status(self) -> CudaStatus:
        if self._handle:
            return _status(_lib.lib().hmp_stitcher_status(self._handle))
        return self._status

    def canvas_width(self) -> int:
        return int(_lib.lib().hmp_stitcher_canvas_width(self._handle)) if self._handle else 0

    def canvas_height(self) -> int:
        return int(_lib.lib().hmp_stitcher_canvas_height(self._handle)) if self._handle else 0

    def batch_size(self) -> int:
        return self._batch

    def info(self) -> dict:
        inf = StitcherInfo()
        _lib.lib().hmp_stitcher_get_info(self._handle, C.byref(inf))
        return {
            "canvas": (inf.canvas_width, inf.canvas_height),
            "levels": inf.levels,
            "blend_rect": tuple(inf.blend_rect),
            "write_rect": tuple(inf.write_rect),
            "tile_down": inf.tile_down,
            "tile_coarse": inf.tile_coarse,
            "launches_per_process": inf.launches_per_process,
            "m0_bytes": inf.m0_bytes,
            "device_bytes": inf.device_bytes,
            "copy_mode": bool(inf.copy_mode),
            "copy_blocks": inf.copy_blocks,
            "empty_blocks": inf.empty_blocks,
            "pyramid_blocks": inf.pyramid_blocks,
            "pyramid_tiles": tuple(inf.pyramid_tiles),
            "gather_pixels": inf.gather_pixels,
        }

    def set_tiles(self, tile_down: int, tile_coarse: int = 32) -> None:
        """Pyramid tile edges (tuning only: every choice gives the same bits)."""
        s = _status(_lib.lib().hmp_stitcher_set_tiles(self._handle, int(tile_down), int(tile_coarse)))
        if not s.ok():
            raise CudaStatusError(s)

    def set_down_residency(self, ctas_per_sm: int) -> None:
        """Caps the Gaussian-pyramid kernel at ctas_per_sm CTAs per SM (0 = no cap); tuning only."""
        s = _status(_lib.lib().hmp_stitcher_set_down_residency(self._handle, int(ctas_per_sm)))
        if not s.ok():
            raise CudaStatusError(s)

    def set_copy_blocks(self, enable: bool, opaque_frames: bool = False) -> None:
        """Copy blocks on (default) or off (both give the same bits). ``opaque_frames``: the caller
        promises every source pixel has alpha != 0 (camera and video frames), which drops the
        per-call alpha check and its fallback launch."""
        mode = (2 if opaque_frames else 1) if enable else 0
        s = _status(_lib.lib().hmp_stitcher_set_copy_blocks(self._handle, mode))
        if not s.ok():
            raise CudaStatusError(s)

    def set_timing(self, enable: bool, serialize: bool = False) -> None:
        """Record per-kernel CUDA-event times of subsequent process() calls; ``serialize`` also runs
        the kernels one after another on the caller stream, so each time is the kernel alone."""
        mode = (2 if serialize else 1) if enable else 0
        s = _status(_lib.lib().hmp_stitcher_set_timing(self._handle, mode))
        if not s.ok():
            raise CudaStatusError(s)

    def kernel_times(self) -> dict:
        """{kernel: (total_ms, launches)} since timing was enabled or last read."""
        t = _lib.KernelTiming()
        s = _status(_lib.lib().hmp_stitcher_get_timing(self._handle, C.byref(t)))
        if not s.ok():
            raise CudaStatusError(s)
        names = ("canvas_gather", "pyr_down", "pyr_coarse", "pyr_fine")
        return {names[i]: (float(t.total_ms[i]), int(t.launches[i])) for i in range(4)}

    def _run(self, inputs: Sequence, canvas=None, stream=None):
        import torch

        st = self.status
        if not st.ok():
            raise CudaStatusError(st)
        _check_backend(getattr(self, "_backend", "auto"))
        batched = [_ensure_batched(t) for t in inputs]
        if any(t.shape[0] != self._batch for t in batched):
            raise ValueError("Input batch size does not match stitcher batch size")
        if any(t.shape[-1] not in (3, 4) for t in batched):
            raise ValueError("Only 3- and 4-channel inputs are supported")
        ptype = _pixel_type(batched[0])
        if any(_pixel_type(t) != ptype for t in batched):
            raise ValueError("inputs must share one pixel type")
        handle = self._handle_for(*ptype)
        device = batched[0].device
        if canvas is None:
            canvas = torch.empty((self._batch, self.canvas_height(), self.canvas_width(), ptype[0]),
                                 dtype=torch.float32 if ptype[1] else torch.uint8, device=device)
        else:
            canvas = _ensure_batched(canvas)
            if canvas.shape[0] != self._batch:
                raise ValueError("Canvas batch size does not match stitcher batch size")
            if _pixel_type(canvas) != ptype:
                raise ValueError("canvas pixel type must match the inputs'")
        imgs = (Image * len(batched))(*[_image(t) for t in batched])
        cv = _image(canvas)
        # The library checks that the current device is the stitcher's; the tensors must live there
        # too (a pointer into another GPU's memory would be read by this GPU's kernels).
        current = torch.cuda.current_device()
        if any(t.device.index != current for t in [*batched, canvas]):
            raise ValueError(f"inputs and canvas must be on the current CUDA device (cuda:{current})")
        if stream is None:
            stream = torch.cuda.current_stream(device).cuda_stream
        elif hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        s = _lib.lib().hmp_stitcher_process(handle, imgs, len(batched), C.byref(cv), C.c_void_p(stream))
        status = _status(s)
        if not status.ok():
            raise CudaStatusError(status)
        self._last_handle = handle  # the dump reads the stitcher of the last call's pixel type
        return canvas


def _check_backend(backend) -> None:
    """The reference's backend names (cupano/ops.py:24, 60-69): "auto" and "triton" select its GPU
    kernels; here both run this library's CUDA kernels, the only backend. Anything else is the
    reference's ValueError, raised by process() as there."""
    if backend not in ("auto", "triton"):
        raise ValueError(f"Unsupported backend: {backend}")


class CudaStitchPano(_Stitcher):
    """Two-image stitcher (src/pano/cudaPano.h:68-115, cupano/pano.py:127-551).

    ``backend`` and ``enable_cuda_graphs`` are the reference Python class's arguments: every
    backend name it accepts runs this library's kernels, and process() launches at most four
    kernels with no allocation, so callers capture it in a CUDA graph themselves if they want one
    (it is capturable from the first call)."""

    _kind = _lib.KIND_PANO2

    def __init__(self, batch_size: int, num_levels: int, control_masks: ControlMasks, quiet: bool = False,
                 minimize_blend: bool = True, max_output_width: int = 0, backend: str = "auto",
                 enable_cuda_graphs: bool = True, *, storage: str = "f32", filter: str = "refbox"):
        del max_output_width, enable_cuda_graphs
        self._backend = backend
        super().__init__(control_masks, num_levels, batch_size, quiet, minimize_blend, True, storage, filter)

    def process(self, input_image_1, input_image_2, canvas=None, stream=None):
        return self._run([input_image_1, input_image_2], canvas, stream)

    def dump_soft_blend_pyramid(self, directory, *, device=None, channels=None, stream=None) -> None:
        """Write the soft-blend pyramid of the last process() under `directory`
        (cupano/pano.py:466-551, src/pano/cudaPano.inl:420-458): metadata.txt and float32 TIFF
        files gauss1 / gauss2 / lap1 / lap2 / blend / reconstruct `level_<l>_batch_<b>.tiff` and
        mask `level_<l>.tiff`, for the pixel type of the last process() (RGBA: uint8 or float).
        The last call's input tensors must still hold their frames. `device` and `channels` are
        accepted for the reference's signature (one device, RGBA)."""
        import torch

        del device, channels
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        elif hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        handle = getattr(self, "_last_handle", None) or self._handle
        s = _status(_lib.lib().hmp_stitcher_dump_pyramid(handle, str(directory).encode(), C.c_void_p(stream)))
        if not s.ok():
            raise CudaStatusError(s)


class CudaStitchPano3(_Stitcher):
    """Three-image stitcher (src/pano/cudaPano3.h:64-182). ``fused`` picks the reference's fused
    remap (invalid table entries leave pixels transparent) or its legacy remap+copy path."""

    _kind = _lib.KIND_PANO3

    def __init__(self, batch_size: int, num_levels: int, control_masks: ControlMasks3, quiet: bool = False,
                 fused: bool = True, *, storage: str = "f32", filter: str = "refbox"):
        super().__init__(control_masks, num_levels, batch_size, quiet, True, fused, storage, filter)

    def process(self, input_image_0, input_image_1, input_image_2, canvas=None, stream=None, fused=None):
        """``fused`` (default: the constructor's) picks the remap per call, as the reference's
        process(..., fused) does (src/pano/cudaPano3.h:101-107); the other mode runs on a second
        stitcher made on first use."""
        inputs = [input_image_0, input_image_1, input_image_2]
        masks, levels, batch, _, ctor_fused, storage, filt = self._args
        if fused is None or bool(fused) == bool(ctor_fused):
            return self._run(inputs, canvas, stream)
        other = getattr(self, "_other_mode", None)
        if other is None:
            other = self._other_mode = CudaStitchPano3(batch, levels, masks, True, bool(fused), storage=storage,
                                                       filter=filt)
        return other._run(inputs, canvas, stream)


class CudaStitchPanoN(_Stitcher):
    """N-image stitcher, N in [2, 8] (src/pano/cudaPanoN.h:80-146, cupano/pano.py:553-911)."""

    _kind = _lib.KIND_PANON

    def __init__(self, batch_size: int, num_levels: int, control_masks: ControlMasksN, quiet: bool = False,
                 minimize_blend: bool = True, backend: str = "auto", enable_cuda_graphs: bool = True, *,
                 storage: str = "f32", filter: str = "refbox"):
        del enable_cuda_graphs  # as for CudaStitchPano
        self._backend = backend
        self._n = len(control_masks.img_col)
        if control_masks.is_valid() and not 2 <= self._n <= 8:
            self._handle = C.c_void_p()
            self._batch = int(batch_size)
            self._status = CudaStatus(1, "Unsupported N for blend (supported 2..8)")
            return
        super().__init__(control_masks, num_levels, batch_size, quiet, minimize_blend, True, storage, filter)

    def process(self, inputs: Iterable, canvas=None, stream=None):
        inputs = list(inputs)
        if len(inputs) != self._n:
            raise ValueError("inputs size != N")
        return self._run(inputs, canvas, stream)


def plan_geometry(kind: int, control_masks, num_levels: int, minimize_blend: bool = True) -> dict:
    """Host-only geometry of a configuration (no GPU needed)."""
    cfg, keep = build_config(kind, control_masks, num_levels, 1, minimize_blend)
    cw, ch = C.c_int(), C.c_int()
    out = (C.c_int * 9)()
    s = _lib.lib().hmp_plan_geometry(C.byref(cfg), C.byref(cw), C.byref(ch), out)
    del keep
    st = _status(s)
    if not st.ok():
        raise CudaStatusError(st)
    v = list(out)
    return {"canvas": (cw.value, ch.value), "blend": tuple(v[0:4]), "write": tuple(v[4:8]), "levels": v[8]}


def plan_copy_blocks(kind: int, control_masks, num_levels: int, minimize_blend: bool = True) -> dict:
    """Host-only copy-block classes of a configuration (hmp_plan_copy_blocks): the canvas origin
    and counts of its 64 x 16 blocks and a [ny, nx] uint8 array, 0 = copy, 1 = pyramid, 2 = empty
    (None when the configuration has no copy blocks)."""
    import numpy as np

    cfg, keep = build_config(kind, control_masks, num_levels, 1, minimize_blend)
    grid = (C.c_int * 4)()
    st = _status(_lib.lib().hmp_plan_copy_blocks(C.byref(cfg), grid, None, 0))
    if not st.ok():
        raise CudaStatusError(st)
    x0, y0, nx, ny = list(grid)
    classes = None
    if nx and ny:
        classes = np.zeros((ny, nx), dtype=np.uint8)
        st = _status(_lib.lib().hmp_plan_copy_blocks(C.byref(cfg), grid, classes.ctypes.data_as(C.c_void_p),
                                                     classes.size))
        if not st.ok():
            raise CudaStatusError(st)
    del keep
    return {"origin": (x0, y0), "blocks": (nx, ny), "classes": classes}


class StitchServer:
    """Continuous-batching stitch server over hmp_server_* (include/hmpano.h).

    Register configurations first (``add_config``), then ``submit`` requests from any thread;
    ``wait`` / ``drain`` return their statuses. Input and canvas tensors are kept referenced here
    until their request finished.
    """

    def __init__(self, hbm_budget_bytes: int, slots: int = 4, max_instances_per_config: int = 2):
        self._h = C.c_void_p()
        opt = _lib.ServerOptions(int(hbm_budget_bytes), int(slots), int(max_instances_per_config))
        st = _status(_lib.lib().hmp_server_create(C.byref(opt), C.byref(self._h)))
        if not st.ok():
            raise CudaStatusError(st)
        self._live = {}
        self._canvas = {}

    def close(self) -> None:
        if self._h:
            _lib.lib().hmp_server_destroy(self._h)
            self._h = C.c_void_p()
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_config(self, kind: int, control_masks, num_levels: int, batch_size: int = 1, minimize_blend: bool = True,
                   fused: bool = True, storage: str = "f32", filter: str = "refbox") -> int:
        cfg, keep = build_config(kind, control_masks, num_levels, batch_size, minimize_blend, fused, storage, filter)
        cid = C.c_int()
        st = _status(_lib.lib().hmp_server_add_config(self._h, C.byref(cfg), C.byref(cid)))
        del keep
        if not st.ok():
            raise CudaStatusError(st)
        return int(cid.value)

    def submit(self, config_id: int, inputs: Sequence, canvas) -> int:
        batched = [_ensure_batched(t) for t in inputs]
        canvas = _ensure_batched(canvas)
        imgs = (Image * len(batched))(*[_image(t) for t in batched])
        cv = _image(canvas)
        rid = C.c_longlong()
        st = _status(_lib.lib().hmp_server_submit(self._h, int(config_id), imgs, len(batched), C.byref(cv),
                                                  C.byref(rid)))
        if not st.ok():
            raise CudaStatusError(st)
        self._live[int(rid.value)] = (batched, canvas)
        return int(rid.value)

    def wait(self, request_id: int, timeout_ms: int = 60000) -> CudaStatus:
        st = _status(_lib.lib().hmp_server_wait(self._h, int(request_id), int(timeout_ms)))
        if st.code != 909:
            self._live.pop(int(request_id), None)
        return st

    def drain(self, timeout_ms: int = 600000) -> CudaStatus:
        st = _status(_lib.lib().hmp_server_drain(self._h, int(timeout_ms)))
        if st.ok():
            self._live.clear()
        return st

    def stats(self) -> dict:
        s = _lib.ServerStats()
        _lib.lib().hmp_server_get_stats(self._h, C.byref(s))
        return {name: getattr(s, name) for name, _ in _lib.ServerStats._fields_}

    def reset_stats(self) -> None:
        _lib.lib().hmp_server_reset_stats(self._h)
