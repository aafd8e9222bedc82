"""``cupano.masks`` names (the reference's cupano/masks.py): this library's control masks."""
from hmpano import UNMAPPED_POSITION_VALUE, ControlMasks, ControlMasks3, ControlMasksN

__all__ = ["ControlMasks", "ControlMasks3", "ControlMasksN", "UNMAPPED_POSITION_VALUE"]
