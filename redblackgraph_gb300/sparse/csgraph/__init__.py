"""GPU drop-in for ``redblackgraph.sparse.csgraph``'s closure functions."""
from ._shortest_path import shortest_path, floyd_warshall, validate_graph
from .transitive_closure import (
    transitive_closure,
    transitive_closure_floyd_warshall,
    transitive_closure_dijkstra,
    transitive_closure_squaring,
    transitive_closure_dag_sparse,
    component_wise_closure,
    transitive_closure_adaptive,
    find_components,
    find_components_sparse,
    get_component_vertices,
    DensificationError,
)
from .cycleerror import CycleError
from ._relational_composition import vertex_relational_composition, edge_relational_composition
from ._components import extract_submatrix, merge_component_matrices
from ._ordering import (avos_canonical_ordering, _get_permutation, _get_permutation_sparse, permute,
                        permute_sparse, topological_sort, topological_ordering, is_upper_triangular)

__all__ = ["shortest_path", "floyd_warshall", "transitive_closure",
           "transitive_closure_floyd_warshall", "transitive_closure_dijkstra",
           "transitive_closure_squaring", "transitive_closure_dag_sparse", "component_wise_closure",
           "transitive_closure_adaptive", "find_components", "find_components_sparse",
           "get_component_vertices", "DensificationError", "CycleError",
           "vertex_relational_composition", "edge_relational_composition",
           "avos_canonical_ordering", "_get_permutation", "_get_permutation_sparse", "permute", "permute_sparse",
           "topological_sort", "topological_ordering", "is_upper_triangular", "extract_submatrix",
           "merge_component_matrices"]
