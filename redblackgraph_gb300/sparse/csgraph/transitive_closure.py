"""Closure entry points of ``redblackgraph.sparse.csgraph`` (transitive_closure.py:17-82)."""
from __future__ import annotations

from ...types import TransitiveClosure
from ._shortest_path import shortest_path


def transitive_closure(R, method="D", assume_upper_triangular=False) -> TransitiveClosure:
    return TransitiveClosure(*shortest_path(R, method=method, directed=True, overwrite=False,
                                            assume_upper_triangular=assume_upper_triangular))


def transitive_closure_floyd_warshall(R, assume_upper_triangular=False) -> TransitiveClosure:
    return transitive_closure(R, method="FW", assume_upper_triangular=assume_upper_triangular)


def transitive_closure_dijkstra(R) -> TransitiveClosure:
    import scipy.sparse as sp
    if sp.issparse(R):
        csr = R.tocsr()
        rows = csr.indptr
        if all((csr.indices[rows[i]:rows[i + 1]] >= i).all() for i in range(csr.shape[0])):
            return transitive_closure_floyd_warshall(R, assume_upper_triangular=True)
    return transitive_closure(R, method="D")
