"""Floyd-Warshall closure of ``redblackgraph.sparse.csgraph`` on the GPU.

Mirrors redblackgraph/sparse/csgraph/_shortest_path.pyx:36-389: the input is validated to a
dense int32 ``rb.array`` (_validation.py:11-60), then closed with the Cython semantics
(signed non-zero minimum, silent wrap, CycleError at the first cycle) by ``rbg_fw_dense`` in
RBG_MODE_CYTHON.  ``assume_upper_triangular`` selects the i <= k <= j loop (:365-378).

The shortest-path methods 'D', 'BF', 'J' and 'auto' (Dijkstra / Bellman-Ford / Johnson in the
reference) return the same closure W for acyclic graphs; here they run the same GPU closure and
report their diameter definition -- MSB of the largest final value (_shortest_path.pyx:842-845).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from ... import _lib
from ...core.redblack import array as rb_array
from ...dense import fw_dense, raise_for_cython
from ...device import require_cuda, to_device, to_host

DTYPE = np.int32


def validate_graph(csgraph, directed=True, dtype=DTYPE, csr_output=False, copy_if_dense=False):
    """Dense int32 ``rb.array`` view of a dense or sparse graph (_validation.py:11-60)."""
    if sp.issparse(csgraph):
        g = np.asarray(csgraph.toarray()).astype(dtype)
    else:
        g = np.array(csgraph, copy=True).astype(dtype)
    if g.ndim != 2:
        raise ValueError("compressed-sparse graph must be 2-D")
    if g.shape[0] != g.shape[1]:
        raise ValueError("compressed-sparse graph must be shape (N, N)")
    return g.view(rb_array)


def _fw(dist: np.ndarray, assume_upper_triangular: bool, final_max: bool = False):
    n = dist.shape[0]
    if n == 0:
        return dist, 0
    dev = require_cuda()
    d = to_device(np.ascontiguousarray(dist), dev)
    mode = _lib.MODE_CYTHON | (_lib.MODE_TRIANGULAR if assume_upper_triangular else 0)
    out, res = fw_dense(d, out=d, mode=mode)
    raise_for_cython(res)
    diameter = int(res.diameter)
    if final_max:
        mx = int(out.max().item())
        diameter = mx.bit_length() - 1 if mx > 1 else 0
    return to_host(out).view(type(dist)), diameter


def floyd_warshall(csgraph, directed=True, return_predecessors=False, unweighted=False,
                   overwrite=False, assume_upper_triangular=False):
    dist = validate_graph(csgraph, directed, DTYPE, csr_output=False, copy_if_dense=not overwrite)
    if unweighted:
        dist[dist != 0] = 1
    dist, diameter = _fw(dist, assume_upper_triangular)
    if return_predecessors:
        return dist, np.full(dist.shape, -9999, dtype=np.int32), diameter
    return dist, diameter


def shortest_path(csgraph, method="auto", directed=True, return_predecessors=False,
                  unweighted=False, overwrite=False, indices=None, assume_upper_triangular=False):
    if method not in ("auto", "FW", "D", "BF", "J"):
        raise ValueError("unrecognized method '%s'" % method)
    if method == "FW":
        return floyd_warshall(csgraph, directed, return_predecessors=return_predecessors,
                              unweighted=unweighted, overwrite=overwrite,
                              assume_upper_triangular=assume_upper_triangular)
    if indices is not None:
        raise NotImplementedError("single-source shortest paths are not on the closure path")
    dist = validate_graph(csgraph, directed, DTYPE, csr_output=False, copy_if_dense=True)
    if unweighted:
        dist[dist != 0] = 1
    dist, diameter = _fw(dist, False, final_max=True)
    if return_predecessors:
        return dist, np.full(dist.shape, -9999, dtype=np.int32), diameter
    return dist, diameter
