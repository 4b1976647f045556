"""redblackgraph_gb300 -- AVOS-semiring transitive closure on NVIDIA GB300 (sm_103a).

A drop-in for the closure path of rappdw/redblackgraph: ``array`` (dense, ``@`` and
``transitive_closure``), ``warshall``, ``sparse.csgraph`` closures and the ``gpu`` sparse API,
computed by hand-written CUDA kernels in ``librbg_gb300.so`` (C ABI: include/rbg_gb300.h).
"""
from .constants import RED_ONE, BLACK_ONE, red_one_for_dtype, black_one_for_dtype, is_red_one, is_black_one
from .types import TransitiveClosure, Color
from .core import array, warshall, transitive_closure, einsum, avos_sum, avos_product
from . import sparse

__version__ = "0.1.0"
__all__ = ["RED_ONE", "BLACK_ONE", "red_one_for_dtype", "black_one_for_dtype", "is_red_one",
           "is_black_one", "TransitiveClosure", "Color", "array", "warshall",
           "transitive_closure", "einsum", "avos_sum", "avos_product", "sparse"]
