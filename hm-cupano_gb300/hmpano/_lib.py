"""ctypes declarations of the C ABI in include/hmpano.h (libhmpano.so).

The library is loaded from this package's ``lib/`` directory (built in-tree by build.py). There is
no fallback: if the library is missing the import of the stitcher classes fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parents[1]
LIB_PATH = Path(os.environ.get("HMPANO_LIB", PKG_ROOT / "lib" / "libhmpano.so"))

KIND_PANON = 1
KIND_PANO2 = 2
KIND_PANO3 = 3
PIXEL_U8 = 0
PIXEL_F32 = 1
STORAGE_F32 = 0
STORAGE_F16 = 1
FILTER_REFBOX = 0
FILTER_BINOMIAL5 = 1


class Status(C.Structure):
    _fields_ = [("code", C.c_int), ("message", C.c_char * 252)]


class Remap(C.Structure):
    _fields_ = [
        ("map_x", C.POINTER(C.c_uint16)),
        ("map_y", C.POINTER(C.c_uint16)),
        ("width", C.c_int),
        ("height", C.c_int),
        ("xpos", C.c_int),
        ("ypos", C.c_int),
    ]


class Config(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("n_images", C.c_int),
        ("num_levels", C.c_int),
        ("batch_size", C.c_int),
        ("channels", C.c_int),
        ("minimize_blend", C.c_int),
        ("fused", C.c_int),
        ("storage", C.c_int),
        ("filter", C.c_int),
        ("remaps", C.POINTER(Remap)),
        ("seam", C.POINTER(C.c_uint8)),
        ("seam_width", C.c_int),
        ("seam_height", C.c_int),
        ("pixel_format", C.c_int),
    ]


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("pitch", C.c_size_t)]


class StitcherInfo(C.Structure):
    _fields_ = [
        ("canvas_width", C.c_int),
        ("canvas_height", C.c_int),
        ("batch_size", C.c_int),
        ("n_images", C.c_int),
        ("levels", C.c_int),
        ("blend_rect", C.c_int * 4),
        ("write_rect", C.c_int * 4),
        ("tile_down", C.c_int),
        ("tile_coarse", C.c_int),
        ("launches_per_process", C.c_int),
        ("m0_bytes", C.c_double),
        ("device_bytes", C.c_double),
        ("copy_mode", C.c_int),
        ("copy_blocks", C.c_int),
        ("empty_blocks", C.c_int),
        ("pyramid_blocks", C.c_int),
        ("pyramid_tiles", C.c_int * 3),
        ("gather_pixels", C.c_double),
    ]


class KernelTiming(C.Structure):
    _fields_ = [("total_ms", C.c_double * 4), ("launches", C.c_longlong * 4)]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("slots", C.c_int), ("max_instances_per_config", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_longlong),
        ("completed", C.c_longlong),
        ("failed", C.c_longlong),
        ("instances_created", C.c_longlong),
        ("instances_evicted", C.c_longlong),
        ("max_in_flight", C.c_int),
        ("p50_ms", C.c_double),
        ("p99_ms", C.c_double),
        ("mean_ms", C.c_double),
        ("max_ms", C.c_double),
        ("span_ms", C.c_double),
        ("canvas_mpix", C.c_double),
        ("resident_bytes", C.c_double),
        ("resident_bytes_peak", C.c_double),
    ]


class ControlDir(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("n", C.c_int),
        ("map_width", C.c_int * 8),
        ("map_height", C.c_int * 8),
        ("map_x", C.POINTER(C.c_uint16) * 8),
        ("map_y", C.POINTER(C.c_uint16) * 8),
        ("xpos", C.c_float * 8),
        ("ypos", C.c_float * 8),
        ("seam_width", C.c_int),
        ("seam_height", C.c_int),
        ("seam", C.POINTER(C.c_uint8)),
        ("internal", C.c_void_p),
    ]


class StabilizeInfo(C.Structure):
    _fields_ = [
        ("corners", C.c_int),
        ("kept", C.c_int),
        ("dx", C.c_float),
        ("dy", C.c_float),
        ("shift_x", C.c_int),
        ("shift_y", C.c_int),
    ]


# Every symbol include/hmpano.h declares, with its signature.
SIGNATURES = {
    "hmp_version": ([], C.c_char_p),
    "hmp_stitcher_create": ([C.POINTER(Config), C.POINTER(C.c_void_p)], Status),
    "hmp_stitcher_destroy": ([C.c_void_p], None),
    "hmp_stitcher_status": ([C.c_void_p], Status),
    "hmp_stitcher_canvas_width": ([C.c_void_p], C.c_int),
    "hmp_stitcher_canvas_height": ([C.c_void_p], C.c_int),
    "hmp_stitcher_batch_size": ([C.c_void_p], C.c_int),
    "hmp_stitcher_get_info": ([C.c_void_p, C.POINTER(StitcherInfo)], Status),
    "hmp_stitcher_process": ([C.c_void_p, C.POINTER(Image), C.c_int, C.POINTER(Image), C.c_void_p], Status),
    "hmp_stitcher_set_timing": ([C.c_void_p, C.c_int], Status),
    "hmp_stitcher_set_tiles": ([C.c_void_p, C.c_int, C.c_int], Status),
    "hmp_stitcher_set_copy_blocks": ([C.c_void_p, C.c_int], Status),
    "hmp_laplacian_rgba": ([C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                            C.c_void_p], Status),
    "hmp_debug_fail_allocation": ([C.c_longlong], None),
    "hmp_debug_allocation_count": ([], C.c_longlong),
    "hmp_stitcher_set_down_residency": ([C.c_void_p, C.c_int], Status),
    "hmp_stitcher_dump_pyramid": ([C.c_void_p, C.c_char_p, C.c_void_p], Status),
    "hmp_stitcher_get_timing": ([C.c_void_p, C.POINTER(KernelTiming)], Status),
    "hmp_plan_geometry": ([C.POINTER(Config), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)], Status),
    "hmp_plan_copy_blocks": ([C.POINTER(Config), C.POINTER(C.c_int), C.c_void_p, C.c_size_t], Status),
    "hmp_server_create": ([C.POINTER(ServerOptions), C.POINTER(C.c_void_p)], Status),
    "hmp_server_destroy": ([C.c_void_p], None),
    "hmp_server_add_config": ([C.c_void_p, C.POINTER(Config), C.POINTER(C.c_int)], Status),
    "hmp_server_submit": ([C.c_void_p, C.c_int, C.POINTER(Image), C.c_int, C.POINTER(Image), C.POINTER(C.c_longlong)],
                          Status),
    "hmp_server_wait": ([C.c_void_p, C.c_longlong, C.c_int], Status),
    "hmp_server_drain": ([C.c_void_p, C.c_int], Status),
    "hmp_server_get_stats": ([C.c_void_p, C.POINTER(ServerStats)], Status),
    "hmp_server_reset_stats": ([C.c_void_p], None),
    "hmp_blend2_noalloc": ([C.POINTER(Image), C.POINTER(Image), C.c_void_p, C.c_size_t, C.c_int, C.c_int,
                            C.POINTER(Image), C.c_void_p], Status),
    "hmp_control_dir_load": ([C.c_char_p, C.c_int, C.c_int, C.POINTER(C.POINTER(ControlDir))], Status),
    "hmp_control_dir_free": ([C.POINTER(ControlDir)], None),
    "hmp_read_seam_png": ([C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p,
                           C.c_size_t], Status),
    "hmp_read_tiff_u16": ([C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_size_t], Status),
    "hmp_batch_create": ([C.POINTER(C.c_void_p)], Status),
    "hmp_batch_destroy": ([C.c_void_p], None),
    "hmp_batch_add": ([C.c_void_p, C.c_void_p, C.POINTER(Image), C.c_int, C.POINTER(Image), C.c_int], Status),
    "hmp_batch_capture": ([C.c_void_p, C.c_void_p], Status),
    "hmp_batch_launch": ([C.c_void_p, C.c_void_p], Status),
    "hmp_stabilizer_create": ([C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)], Status),
    "hmp_stabilizer_destroy": ([C.c_void_p], None),
    "hmp_stabilizer_corners": ([C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_void_p], Status),
    "hmp_stabilizer_flow": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], Status),
    "hmp_stabilizer_warp": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], Status),
    "hmp_stabilizer_run": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_int,
                            C.c_void_p], Status),
    "hmp_stabilizer_get_features": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(StabilizeInfo),
                                     C.c_void_p], Status),
    "hmp_stabilizer_get_response": ([C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p], Status),
    "hmp_stabilizer_set_features": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], Status),
}

NOALLOC_SCRATCH_BYTES = 48 * 1024 * 1024  # HMP_NOALLOC_SCRATCH_BYTES

_lib = None


def lib() -> C.CDLL:
    """Load libhmpano.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"libhmpano.so not found at {LIB_PATH}; run hm-cupano_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib
