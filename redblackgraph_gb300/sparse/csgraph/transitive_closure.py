"""Closure entry points of ``redblackgraph.sparse.csgraph`` (transitive_closure.py:17-574)."""
from __future__ import annotations

import numpy as np

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


# ------------------------------------------------------------------------- sparse closures
def _is_upper(csr) -> bool:
    rows = np.repeat(np.arange(csr.shape[0]), np.diff(csr.indptr))
    return bool(np.all(csr.indices >= rows))


def _is_lower(csr) -> bool:
    rows = np.repeat(np.arange(csr.shape[0]), np.diff(csr.indptr))
    return bool(np.all(csr.indices <= rows))


def _as_csr(A):
    import scipy.sparse as sp
    if not sp.issparse(A):
        return sp.csr_matrix(A)
    return A.tocsr() if not isinstance(A, sp.csr_matrix) else A


def _squaring(csr, max_iterations, cycle_error, dag_candidates=False):
    """R <- R (+) R^2 on the GPU until R is stable; returns (rb_matrix int32, max |value|)."""
    import torch
    from ...spgemm import DeviceCSR, squaring_closure, SEM_C64
    from ... import _lib
    from ..rbm import rb_matrix
    a = csr.copy()
    a.sort_indices()
    a.sum_duplicates()
    if a.dtype.kind not in "iu":
        a = a.astype(np.int64)
    if a.dtype.itemsize < 4:
        a = a.astype(np.int32 if a.dtype.kind == "i" else np.uint32)

    def on_step(rc, flags):
        if cycle_error and (flags & _lib.EV_CYCLE):
            from .cycleerror import CycleError
            raise CycleError("Graph contains a cycle", vertex=-1)
        if rc == _lib.RBG_ERR_OVERFLOW:
            raise OverflowError("Avos product results in an overflow.")

    R, _ = squaring_closure(DeviceCSR.from_scipy(a), max_iterations, SEM_C64, on_step=on_step)
    if R.data.dtype != torch.int32:
        R = DeviceCSR(R.indptr, R.indices, R.data.to(torch.int32), R.shape)
    mx_abs = int(R.data.abs().max().item()) if R.nnz else 0
    mx = int(R.data.max().item()) if R.nnz else 0
    if dag_candidates:
        mx = _dag_candidate_max(a, R)
    return R.to_scipy(cls=rb_matrix), mx_abs, mx


def _dag_candidate_max(a, C):
    """Largest magnitude among A's entries and the candidates A[v][w] (x) C[w][x] (w != v) that
    the reference's DAG closure examines (_transitive_closure_dag.pyx:262-305)."""
    import ctypes
    import torch
    from ...spgemm import DeviceCSR
    from ... import _lib
    from ...device import stream_handle
    A = DeviceCSR.from_scipy(a, dtype=np.int32)
    ws = torch.empty(256, dtype=torch.uint8, device=C.indptr.device)
    out = ctypes.c_int64(0)
    L = _lib.load()
    ca, cc = A.cstruct(), C.cstruct()
    _lib.check(L.rbg_dag_candidate_max(ctypes.byref(ca), ctypes.byref(cc), ws.data_ptr(), ws.numel(),
                                       ctypes.byref(out), stream_handle()), "dag_candidate_max")
    return int(out.value)


def transitive_closure_dag_sparse(A) -> TransitiveClosure:
    """Closure of a DAG (redblackgraph/sparse/csgraph/transitive_closure.py:383-438): the
    reference's parent-by-parent propagation, run level by level on the GPU (rbg_dag_closure);
    the diameter is the reference's: MSB of the largest magnitude among the input's entries and
    every candidate A[v][w] (x) C[w][x], including candidates that lose the (+)
    (_transitive_closure_dag.pyx:262-305, 347-349); CycleError on a cycle."""
    import scipy.sparse as sp
    from ...dag import RowTooWide, dag_closure_device
    from ...spgemm import DeviceCSR
    from ..rbm import rb_matrix
    csr = _as_csr(A)
    n = csr.shape[0]
    if n == 0:
        return TransitiveClosure(sp.csr_matrix((0, 0), dtype=np.int32), 0)
    a = csr.copy()
    a.sum_duplicates()
    a.sort_indices()
    try:   # by topological levels (the reference's algorithm, level-parallel)
        C, mx, _ = dag_closure_device(DeviceCSR.from_scipy(a, dtype=np.int32))
    except RowTooWide:   # rows past the level kernels' tables: the same closure by squaring
        W, mx_abs, mx = _squaring(csr, 64, cycle_error=True, dag_candidates=True)
        return TransitiveClosure(W, (mx.bit_length() - 1) if mx > 1 else 0)
    return TransitiveClosure(C.to_scipy(cls=rb_matrix), (mx.bit_length() - 1) if mx > 1 else 0)


def transitive_closure_squaring(A, max_iterations=64) -> TransitiveClosure:
    """Closure by repeated squaring (transitive_closure.py:198-269): triangular inputs take the
    DAG closure, others iterate R <- R (+) R^2 with the magnitude merge until stable."""
    import scipy.sparse as sp
    csr = _as_csr(A)
    n = csr.shape[0]
    if n == 0:
        return TransitiveClosure(sp.csr_matrix((0, 0), dtype=np.int32), 0)
    if _is_upper(csr) or _is_lower(csr):
        return transitive_closure_dag_sparse(csr)
    W, mx_abs, _ = _squaring(csr, max_iterations, cycle_error=False)
    diameter = int(np.floor(np.log2(mx_abs))) if mx_abs > 1 else 0
    return TransitiveClosure(W, diameter)


def component_wise_closure(A, method: str = "auto", densify_threshold: int = 500) -> TransitiveClosure:
    """Closure of every connected component separately, merged into one sparse matrix
    (redblackgraph/sparse/csgraph/transitive_closure.py:85-195).

    All components are closed by one batched GPU call; each component's diameter follows the
    method the reference would pick for it ("FW": the Floyd-Warshall running maximum, "D": MSB of
    the largest final value) and the result's diameter is their maximum.  Values are int32
    (the reference's DTYPE); W is a CSR matrix with int32 values and sorted rows.
    """
    import scipy.sparse as sp
    from ...device import csr_from_parts, require_cuda, to_device, to_host_pinned
    from ...components import component_closure_device
    csr = _as_csr(A)
    n = csr.shape[0]
    if n == 0:
        return TransitiveClosure(sp.csr_matrix((0, 0), dtype=np.int32), 0)
    if not csr.has_canonical_format:
        csr = csr.copy()
        csr.sum_duplicates()
    import torch
    dev = require_cuda()
    # index arrays go over as they are and are widened/narrowed on the device; values are cast
    # to int32 on the host first (the reference's np.asarray(A.data, dtype=DTYPE))
    ip = to_device(np.ascontiguousarray(csr.indptr), dev).to(torch.int64)
    ij = to_device(np.ascontiguousarray(csr.indices), dev).to(torch.int32)
    iv = to_device(np.ascontiguousarray(csr.data).astype(np.int32, copy=False), dev)
    oi, oj, ov, diameter, _ = component_closure_device(ip, ij, iv, n, method, densify_threshold)
    if ov.numel() < 2**31 - 1:   # int32 row pointers when they fit: scipy keeps the arrays as given
        oi = oi.to(torch.int32)
    W = csr_from_parts(to_host_pinned(ov), to_host_pinned(oj), to_host_pinned(oi), (n, n))
    return TransitiveClosure(W, int(diameter))


# ------------------------------------------------------------------------- components, dispatch
class DensificationError(Exception):
    """Raised when an operation would densify (redblackgraph/sparse/csgraph/_density.py:14-25)."""

    def __init__(self, message: str, density: float, threshold: float):
        self.density = density
        self.threshold = threshold
        super().__init__(message)


def find_components_sparse(A, q=None) -> np.ndarray:
    """Connected components with edges taken both ways, numbered by least vertex, on the GPU
    (redblackgraph/sparse/csgraph/_components.pyx:86-177).  Returns uint32 labels; fills ``q``
    (component -> vertex count) when given."""
    import torch
    from ...device import require_cuda, to_device, to_host
    from ...components import label_components
    csr = _as_csr(A)
    n = csr.shape[0]
    if n == 0:
        return np.zeros(0, dtype=np.uint32)
    dev = require_cuda()
    ip = to_device(np.ascontiguousarray(csr.indptr), dev).to(torch.int64)
    ij = to_device(np.ascontiguousarray(csr.indices), dev).to(torch.int32)
    comps = label_components(ip, ij, n)
    if q is not None:
        q.clear()
        q.update({c: int(s) for c, s in enumerate(comps.sizes.tolist())})
    return to_host(comps.label[:n]).astype(np.uint32)


def find_components(A, q=None) -> np.ndarray:
    """Components of a dense or sparse graph (_components.pyx:12-83, 86-177)."""
    return find_components_sparse(A, q)


def get_component_vertices(component_labels) -> dict:
    """component id -> its vertices, ascending (_components.pyx:326-344)."""
    lab = np.asarray(component_labels)
    order = np.argsort(lab, kind="stable")
    ids, starts = np.unique(lab[order], return_index=True)
    bounds = list(starts) + [lab.size]
    return {int(c): order[bounds[k]:bounds[k + 1]].astype(np.int32) for k, c in enumerate(ids)}


def transitive_closure_adaptive(A, method: str = "auto", density_threshold: float = 0.1,
                                component_threshold: int = 1, size_threshold: int = 1000,
                                sparse_only: bool = False) -> TransitiveClosure:
    """The reference's strategy selection (redblackgraph/sparse/csgraph/transitive_closure.py:
    441-574) over the GPU closures: several components -> component_wise_closure; very sparse and
    large -> the 'D' closure; triangular -> the DAG closure; otherwise Floyd-Warshall.
    ``sparse_only`` runs the DAG closure and turns a cycle into DensificationError."""
    import scipy.sparse as sp
    from .cycleerror import CycleError
    csr = _as_csr(A)
    n = csr.shape[0]
    if n == 0:
        return TransitiveClosure(sp.csr_matrix((0, 0), dtype=np.int32), 0)
    if sparse_only:
        try:
            return transitive_closure_dag_sparse(csr)
        except CycleError as e:
            raise DensificationError(f"sparse_only=True requires a DAG, but graph contains cycles: {e}",
                                     density=1.0, threshold=0.0)
    if method == "FW":
        return transitive_closure(csr, method="FW")
    if method == "D":
        return transitive_closure(csr, method="D")
    if method == "component":
        return component_wise_closure(csr)
    if method == "squaring":
        return transitive_closure_squaring(csr)
    if method == "dag_sparse":
        return transitive_closure_dag_sparse(csr)
    q = {}
    find_components_sparse(csr, q)
    if len(q) > component_threshold:
        return component_wise_closure(csr)
    density = csr.nnz / (n * n)
    if density < density_threshold and n > size_threshold:
        return transitive_closure(csr, method="D")
    if _is_upper(csr) or _is_lower(csr):
        return transitive_closure_dag_sparse(csr)
    return transitive_closure(csr, method="FW")
