"""Dense AVOS API mirroring redblackgraph.core (redblackgraph/core/__init__.py)."""
from .warshall import warshall
from .avos import einsum, avos_sum, avos_product
from .redblack import array, transitive_closure, vertex_relational_composition, edge_relational_composition

__all__ = ["warshall", "einsum", "avos_sum", "avos_product", "array", "transitive_closure",
           "vertex_relational_composition", "edge_relational_composition"]
