"""Region-model API (``src/mbem/model/__init__.py``)."""

from .core import FAULT_KINDS, FAULT_ORIENTATION, BCType, Patch, Region, RegionModel
from .equations import BlockSystem, BlockTerm, RhsTerm, RhsValue, generate_system
from .layout import Slot, UnknownLayout

__all__ = ["BCType", "Patch", "Region", "RegionModel", "FAULT_KINDS", "FAULT_ORIENTATION",
           "BlockSystem", "BlockTerm", "RhsTerm", "RhsValue", "generate_system", "Slot",
           "UnknownLayout"]
