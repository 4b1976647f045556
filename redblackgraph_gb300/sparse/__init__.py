"""GPU drop-in for ``redblackgraph.sparse``."""
from .csgraph import *  # noqa: F401,F403
from .csgraph import __all__ as _cs_all

__all__ = list(_cs_all)
