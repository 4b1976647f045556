"""CycleError (redblackgraph/sparse/csgraph/cycleerror.py:1-6)."""
from ...dense import CycleError

__all__ = ["CycleError"]
