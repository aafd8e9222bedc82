"""The `cupano` names (hm-cupano_gb300/cupano) on the CPU: everything the reference package exports
imports, and compute_laplacian rejects what the reference rejects before any device work."""
from __future__ import annotations

import pytest


def test_reference_names_import():
    import cupano
    import hmpano
    from cupano.geometry import CanvasInfo, Rect, SpatialTiff
    from cupano.masks import UNMAPPED_POSITION_VALUE, ControlMasks, ControlMasksN
    from cupano.ops import compute_laplacian
    from cupano.pano import CudaStitchPano, CudaStitchPanoN
    from cupano.status import CudaStatus, CudaStatusError

    for name in ("CanvasInfo", "ControlMasks", "ControlMasksN", "CudaStatus", "CudaStatusError", "CudaStitchPano",
                 "CudaStitchPanoN", "Rect", "SpatialTiff", "UNMAPPED_POSITION_VALUE"):
        assert getattr(cupano, name) is getattr(hmpano, name), name
    assert callable(compute_laplacian)
    del CanvasInfo, Rect, SpatialTiff, UNMAPPED_POSITION_VALUE, ControlMasks, ControlMasksN, CudaStitchPano
    del CudaStitchPanoN, CudaStatus, CudaStatusError


def test_compute_laplacian_argument_errors():
    import torch
    from cupano.ops import compute_laplacian

    high = torch.zeros((1, 4, 4, 4))
    low = torch.zeros((1, 2, 2, 4))
    with pytest.raises(ValueError, match="Unsupported backend"):
        compute_laplacian(high, low, backend="torch")
    with pytest.raises(ValueError, match="RGBA"):
        compute_laplacian(torch.zeros((1, 4, 4, 3)), torch.zeros((1, 2, 2, 3)))
