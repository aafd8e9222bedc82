"""hmpano -- GB300-native (sm_103a) implementation of hm-cupano's per-frame stitching path.

The stitch itself runs in libhmpano.so (CUDA kernels behind the C ABI of include/hmpano.h);
this package mirrors the reference's Python/C++ stitcher API on top of it.
"""
from .pano import (
    UNMAPPED_POSITION_VALUE,
    Batch,
    CanvasInfo,
    ControlMasks,
    ControlMasks3,
    ControlMasksN,
    CudaStatus,
    CudaStatusError,
    CudaStitchPano,
    CudaStitchPano3,
    CudaStitchPanoN,
    Rect,
    SpatialTiff,
    StitchServer,
    load_control_dir,
    plan_copy_blocks,
    plan_geometry,
    read_seam_png,
    read_tiff_u16,
)
from .stabilize import Motion, Stabilizer

__all__ = [
    "Batch",
    "CanvasInfo",
    "ControlMasks",
    "ControlMasks3",
    "ControlMasksN",
    "CudaStatus",
    "CudaStatusError",
    "CudaStitchPano",
    "CudaStitchPano3",
    "CudaStitchPanoN",
    "Motion",
    "Rect",
    "SpatialTiff",
    "Stabilizer",
    "StitchServer",
    "UNMAPPED_POSITION_VALUE",
    "load_control_dir",
    "plan_copy_blocks",
    "plan_geometry",
    "read_seam_png",
    "read_tiff_u16",
]
