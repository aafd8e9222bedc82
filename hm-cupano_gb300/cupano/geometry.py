"""``cupano.geometry`` names (the reference's cupano/geometry.py): this library's types."""
from hmpano import CanvasInfo, Rect, SpatialTiff

__all__ = ["CanvasInfo", "Rect", "SpatialTiff"]
