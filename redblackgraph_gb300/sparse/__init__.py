"""GPU drop-in for ``redblackgraph.sparse``."""
from .rbm import rb_matrix
from .csgraph import *  # noqa: F401,F403
from .csgraph import __all__ as _cs_all

__all__ = ["rb_matrix"] + list(_cs_all)
