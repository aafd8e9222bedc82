"""``cupano.pano`` names (the reference's cupano/pano.py): this library's stitchers."""
from hmpano import CudaStitchPano, CudaStitchPano3, CudaStitchPanoN

__all__ = ["CudaStitchPano", "CudaStitchPano3", "CudaStitchPanoN"]
