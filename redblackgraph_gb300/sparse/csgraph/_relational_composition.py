"""``vertex_relational_composition`` / ``edge_relational_composition`` of
redblackgraph.sparse.csgraph (_relational_composition.pyx:10-113): int32 closures, the Cython
algebra (signed non-zero minimum, silent wrap), no cycle check; on the GPU through
``rbg_vertex_compose`` / ``rbg_edge_compose`` with RBG_MODE_CYTHON."""
from __future__ import annotations

import numpy as np

from ...composition import edge_compose_host, vertex_compose_host

__all__ = ["vertex_relational_composition", "edge_relational_composition"]


def _int32(x, what):
    a = np.asarray(x)
    if a.dtype != np.int32:
        raise ValueError(f"Buffer dtype mismatch, expected 'DTYPE_t' but got '{a.dtype.name}' ({what})")
    return a


def vertex_relational_composition(u, R, v, color):
    """R_lambda: the closure with a new vertex (row u, column v, colour ``color``)."""
    R = _int32(R, "R")
    N = R.shape[0]
    assert N == R.shape[1]
    u = _int32(u, "u").reshape((N,))
    v = _int32(v, "v").reshape((N,))
    return vertex_compose_host(u, R, v, int(color), cython=True)


def edge_relational_composition(R, alpha, beta, relationship):
    """R': the closure with the edge alpha -> beta of value ``relationship``."""
    R = _int32(R, "R")
    N = R.shape[0]
    assert N == R.shape[1]
    return edge_compose_host(R, int(alpha), int(beta), int(relationship), cython=True)
