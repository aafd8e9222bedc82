"""``cupano.status`` names (the reference's cupano/status.py): this library's status types."""
from hmpano import CudaStatus, CudaStatusError

__all__ = ["CudaStatus", "CudaStatusError"]
