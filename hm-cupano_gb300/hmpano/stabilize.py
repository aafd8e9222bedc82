"""Frame stabiliser over hmp_stabilizer_* (libhmpano.so): the steps of src/cuda/cudaStabilize.cu.

    harrisCornerDetection(d_img, w, h, k, threshold, corners)   cudaStabilize.cu:157   -> corners()
    computeOpticalFlow(d_prev, d_next, features, flow, ...)      cudaStabilize.cu:210   -> flow()
    stabilizeFrame(d_frame, w, h, flow)                          cudaStabilize.cu:243   -> warp()
    main(): the three in sequence                                cudaStabilize.cu:274   -> run()

Frames are 2-D float32 CUDA tensors (grayscale, contiguous). Every step is asynchronous on the
given stream (default: torch's current stream); features() waits and reads the results back.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .pano import CudaStatusError, _status

HARRIS_K = 0.04      # cudaStabilize.cu:294
THRESHOLD = 1e6      # cudaStabilize.cu:295
WINDOW_SIZE = 15     # cudaStabilize.cu:300


@dataclass(frozen=True)
class Motion:
    corners: int     # corners found in the previous frame
    kept: int        # of them, tracked
    dx: float        # mean flow, next relative to previous
    dy: float
    shift_x: int     # the translation applied (dx, dy rounded)
    shift_y: int


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class Stabilizer:
    """Allocates once for width x height frames and up to max_features tracked corners (0: every
    interior pixel may be one)."""

    def __init__(self, width: int, height: int, max_features: int = 0):
        self.width, self.height = int(width), int(height)
        self._h = C.c_void_p()
        s = _status(_lib.lib().hmp_stabilizer_create(self.width, self.height, int(max_features), C.byref(self._h)))
        if not s.ok():
            raise CudaStatusError(s)
        self.max_features = int(max_features) if max_features else (self.width - 2) * (self.height - 2)

    def _frame(self, t):
        import torch

        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
                and tuple(t.shape) == (self.height, self.width)):
            raise ValueError(f"frames must be contiguous float32 CUDA tensors of shape {(self.height, self.width)}")
        return C.c_void_p(t.data_ptr())

    def _check(self, s):
        s = _status(s)
        if not s.ok():
            raise CudaStatusError(s)

    def corners(self, img, k: float = HARRIS_K, threshold: float = THRESHOLD, stream=None) -> None:
        self._check(_lib.lib().hmp_stabilizer_corners(self._h, self._frame(img), float(k), float(threshold),
                                                      C.c_void_p(_stream(stream))))

    def flow(self, prev, nxt, window_size: int = WINDOW_SIZE, stream=None) -> None:
        self._check(_lib.lib().hmp_stabilizer_flow(self._h, self._frame(prev), self._frame(nxt), int(window_size),
                                                   C.c_void_p(_stream(stream))))

    def warp(self, frame, out=None, stream=None):
        """Translate `frame` by the current motion into `out` (default: in place, as the reference)."""
        out = frame if out is None else out
        self._check(_lib.lib().hmp_stabilizer_warp(self._h, self._frame(frame), self._frame(out),
                                                   C.c_void_p(_stream(stream))))
        return out

    def run(self, prev, nxt, out=None, k: float = HARRIS_K, threshold: float = THRESHOLD,
            window_size: int = WINDOW_SIZE, stream=None):
        out = nxt if out is None else out
        self._check(_lib.lib().hmp_stabilizer_run(self._h, self._frame(prev), self._frame(nxt), self._frame(out),
                                                  float(k), float(threshold), int(window_size),
                                                  C.c_void_p(_stream(stream))))
        return out

    def features(self, stream=None):
        """(xy int32 [kept, 2], flow float32 [kept, 2], Motion), after waiting for `stream`."""
        info = _lib.StabilizeInfo()
        self._check(_lib.lib().hmp_stabilizer_get_features(self._h, None, None, 0, C.byref(info),
                                                           C.c_void_p(_stream(stream))))
        n = int(info.kept)
        xy = np.zeros((max(n, 1), 2), np.int32)
        fl = np.zeros((max(n, 1), 2), np.float32)
        self._check(_lib.lib().hmp_stabilizer_get_features(self._h, xy.ctypes.data_as(C.c_void_p),
                                                           fl.ctypes.data_as(C.c_void_p), n, C.byref(info),
                                                           C.c_void_p(_stream(stream))))
        motion = Motion(int(info.corners), n, float(info.dx), float(info.dy), int(info.shift_x), int(info.shift_y))
        return xy[:n], fl[:n], motion

    def response(self, stream=None) -> np.ndarray:
        """The last Harris response map (float32 [height, width]), after waiting for `stream`."""
        out = np.zeros((self.height, self.width), np.float32)
        self._check(_lib.lib().hmp_stabilizer_get_response(self._h, out.ctypes.data_as(C.c_void_p), out.size,
                                                           C.c_void_p(_stream(stream))))
        return out

    def set_features(self, xy, stream=None) -> None:
        xy = np.ascontiguousarray(xy, dtype=np.int32).reshape(-1, 2)
        self._check(_lib.lib().hmp_stabilizer_set_features(self._h, xy.ctypes.data_as(C.c_void_p), len(xy),
                                                           C.c_void_p(_stream(stream))))

    def close(self) -> None:
        if self._h:
            _lib.lib().hmp_stabilizer_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
