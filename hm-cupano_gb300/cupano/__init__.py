"""The reference's Python package names over this library.

Code written against hm-cupano's ``cupano`` package (cupano/__init__.py; its stitchers in
cupano/pano.py:127-911) imports the same names from here and runs this library's sm_103a kernels:
the stitchers, masks and geometry types are ``hmpano``'s, and ``cupano.ops.compute_laplacian`` is
the library's Laplacian kernel. The reference's Triton and torch fallbacks are not provided: the
backend names "auto" and "triton" select this library's kernels, any other is the reference's
ValueError.
"""
from hmpano import (
    UNMAPPED_POSITION_VALUE,
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
)

from . import geometry, masks, ops, pano, status

__all__ = [
    "CanvasInfo",
    "ControlMasks",
    "ControlMasks3",
    "ControlMasksN",
    "CudaStatus",
    "CudaStatusError",
    "CudaStitchPano",
    "CudaStitchPano3",
    "CudaStitchPanoN",
    "Rect",
    "SpatialTiff",
    "UNMAPPED_POSITION_VALUE",
    "geometry",
    "masks",
    "ops",
    "pano",
    "status",
]
