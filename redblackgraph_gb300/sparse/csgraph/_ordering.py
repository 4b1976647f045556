"""Canonical ordering, permutation and topological sort of graphs on the GPU.

Mirrors redblackgraph.sparse.csgraph's ``avos_canonical_ordering``, ``_get_permutation``,
``_get_permutation_sparse`` (_ordering.pyx:15-177), ``permute``, ``permute_sparse``
(_permutation.pyx:11-205), ``topological_sort``, ``topological_ordering`` and
``is_upper_triangular`` (_topological_sort.pyx:30-265), with the same arguments and results.
The metrics, sorts and permutations run in librbg_gb300.so (``rbg_ordering_metrics_*``,
``rbg_canonical_permutation``, ``rbg_permute_*``, ``rbg_topological_order``,
``rbg_is_upper_triangular_csr``).  ``topological_sort`` returns a topological order by levels
(deepest first) rather than the reference's depth-first order: another permutation with the same
property (the permuted matrix is upper triangular) where several exist.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ... import _lib
from ...device import csr_from_parts, require_cuda, to_device, to_host
from ...spgemm import DeviceCSR
from ...types import Ordering
from .cycleerror import CycleError

__all__ = ["avos_canonical_ordering", "_get_permutation", "_get_permutation_sparse", "permute",
           "permute_sparse", "topological_sort", "topological_ordering", "is_upper_triangular"]


def _isspmatrix(A) -> bool:
    import scipy.sparse as sp
    return sp.issparse(A)


def _csr_int32(A):
    import scipy.sparse as sp
    csr = A.tocsr() if sp.issparse(A) else sp.csr_matrix(np.asarray(A))
    if csr.dtype != np.int32:
        csr = csr.astype(np.int32)
    return csr


def _device_csr(csr) -> DeviceCSR:
    return DeviceCSR.from_scipy(csr, dtype=np.int32)


def _permutation_from_metrics(n, dev, label, comp_start, anc, maxrel, diag) -> np.ndarray:
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_canonical_permutation_workspace_bytes(n, ctypes.byref(nb)), "canonical_permutation")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    perm = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_canonical_permutation(n, label.data_ptr(), comp_start.data_ptr(), anc.data_ptr(),
                                           maxrel.data_ptr(), diag.data_ptr(), perm.data_ptr(), ws.data_ptr(),
                                           ws.numel(), 0), "canonical_permutation")
    return to_host(perm[:n]).astype(np.int32)


def _components_device(ids, q, n, dev):
    """Component labels and size offsets on the device from (ids, q) as the caller gives them."""
    ids = np.asarray(ids).astype(np.int64)
    count = int(ids.max()) + 1 if n else 0
    sizes = np.zeros(count, np.int64)
    for c, s in q.items():
        if 0 <= int(c) < count:
            sizes[int(c)] = int(s)
    start = np.zeros(count + 1, np.int64)
    np.cumsum(sizes, out=start[1:])
    return (to_device(ids.astype(np.int32), dev), to_device(start, dev))


def _canonical(A, q, ids, sparse: bool) -> np.ndarray:
    n = A.shape[0]
    if n == 0:
        return np.zeros(0, np.int32)
    dev = require_cuda()
    L = _lib.load()
    anc = torch.empty(n, dtype=torch.int64, device=dev)
    maxrel = torch.empty(n, dtype=torch.int32, device=dev)
    diag = torch.empty(n, dtype=torch.int32, device=dev)
    if sparse:
        d = _device_csr(_csr_int32(A))
        ip = d.indptr
        _lib.check(L.rbg_ordering_metrics_csr(n, ip.data_ptr(), d.indices.data_ptr() if d.nnz else ip.data_ptr(),
                                              d.data.data_ptr() if d.nnz else ip.data_ptr(), anc.data_ptr(),
                                              maxrel.data_ptr(), diag.data_ptr(), 0), "ordering_metrics")
    else:
        a = np.ascontiguousarray(np.asarray(A), dtype=np.int32)
        da = to_device(a, dev)
        _lib.check(L.rbg_ordering_metrics_dense(n, da.data_ptr(), n, anc.data_ptr(), maxrel.data_ptr(),
                                                diag.data_ptr(), 0), "ordering_metrics")
    label, start = _components_device(ids, q, n, dev)
    return _permutation_from_metrics(n, dev, label, start, anc, maxrel, diag)


def _get_permutation(A, q, ids):
    """Canonical permutation of a dense closure (_ordering.pyx:15-39)."""
    return _canonical(A, q, ids, sparse=False).tolist()


def _get_permutation_sparse(A, q, ids):
    """Canonical permutation of a sparse closure (_ordering.pyx:42-98)."""
    return _canonical(A, q, ids, sparse=True).tolist()


def avos_canonical_ordering(A) -> Ordering:
    """Canonical ordering of a closure: components largest first, then by ancestor count, column
    maximum, colour and vertex id (_ordering.pyx:152-177)."""
    from .transitive_closure import find_components
    q: dict = {}
    components = find_components(A, q)
    if _isspmatrix(A):
        permutation = _canonical(A, q, components, sparse=True)
        return Ordering(permute_sparse(A, permutation), permutation, q)
    permutation = _canonical(A, q, components, sparse=False)
    return Ordering(permute(A, permutation), permutation, q)


def permute(A, p, assume_upper_triangular=False):
    """P A P^-1 for dense or sparse A (_permutation.pyx:11-34)."""
    if _isspmatrix(A):
        return permute_sparse(A, p, assume_upper_triangular)
    return _permute_dense(A, p, assume_upper_triangular)


def _permute_dense(A, p, assume_upper_triangular=False):
    """B[i][j] = A[p[i]][p[j]] (j >= i only when triangular), int32 (_permutation.pyx:37-63)."""
    a = np.ascontiguousarray(np.asarray(A), dtype=np.int32)
    n = a.shape[0]
    pp = np.ascontiguousarray(np.asarray(p), dtype=np.int32)
    if pp.shape[0] != n or a.ndim != 2 or a.shape[1] != n:
        raise AssertionError("permutation and matrix sizes differ")
    if n == 0:
        return np.zeros(a.shape, np.int32)
    dev = require_cuda()
    da, dp = to_device(a, dev), to_device(pp, dev)
    out = torch.empty((n, n), dtype=torch.int32, device=dev)
    _lib.check(_lib.load().rbg_permute_dense(_lib.dtype_code(np.int32), n, da.data_ptr(), n, dp.data_ptr(),
                                             out.data_ptr(), n, 1 if assume_upper_triangular else 0, 0),
               "permute_dense")
    return to_host(out)


def permute_sparse(A, p, assume_upper_triangular=False):
    """Sparse P A P^-1 as CSR with sorted columns (_permutation.pyx:66-205)."""
    import scipy.sparse as sp
    csr = _csr_int32(A)
    n = csr.shape[0]
    pp = np.ascontiguousarray(np.asarray(p), dtype=np.int32)
    if n == 0:
        return sp.csr_matrix((0, 0), dtype=np.int32)
    dev = require_cuda()
    d = _device_csr(csr)
    dp = to_device(pp, dev)
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_permute_csr_workspace_bytes(n, d.nnz, ctypes.byref(nb)), "permute_csr")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    ip = torch.empty(n + 1, dtype=torch.int64, device=dev)
    nnz = ctypes.c_int64(0)
    ca = d.cstruct()
    upper = 1 if assume_upper_triangular else 0
    _lib.check(L.rbg_permute_csr_count(ctypes.byref(ca), dp.data_ptr(), upper, ip.data_ptr(), ws.data_ptr(),
                                       ws.numel(), ctypes.byref(nnz), 0), "permute_csr")
    m = int(nnz.value)
    oj = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    ox = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_permute_csr_fill(ctypes.byref(ca), dp.data_ptr(), upper, ip.data_ptr(), oj.data_ptr(),
                                      ox.data_ptr(), ws.data_ptr(), ws.numel(), 0), "permute_csr")
    return csr_from_parts(to_host(ox[:m]), to_host(oj[:m]), to_host(ip), (n, n))


def topological_sort(A) -> np.ndarray:
    """A permutation p (p[new] = old) after which the graph's matrix is upper triangular;
    CycleError on a cycle (_topological_sort.pyx:30-181)."""
    csr = _csr_int32(A)
    n = csr.shape[0]
    if n == 0:
        return np.array([], dtype=np.int32)
    dev = require_cuda()
    d = _device_csr(csr)
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_topological_workspace_bytes(n, d.nnz, ctypes.byref(nb)), "topological_order")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    levels, cyc = ctypes.c_int64(0), ctypes.c_int64(-1)
    ca = d.cstruct()
    rc = L.rbg_topological_order(ctypes.byref(ca), ws.data_ptr(), ws.numel(), perm.data_ptr(), ctypes.byref(levels),
                                 ctypes.byref(cyc), 0)
    if rc == _lib.RBG_ERR_CYCLE:
        raise CycleError("Graph contains a cycle", vertex=int(cyc.value))
    _lib.check(rc, "topological_order")
    return to_host(perm).astype(np.int32)


def topological_ordering(A) -> Ordering:
    """topological_sort applied: Ordering(upper triangular matrix, permutation, component sizes)
    (_topological_sort.pyx:184-229)."""
    from .transitive_closure import find_components
    perm = topological_sort(A)
    q: dict = {}
    find_components(A, q)
    if _isspmatrix(A):
        return Ordering(permute_sparse(A, perm, assume_upper_triangular=True), perm, q)
    return Ordering(permute(A, perm, assume_upper_triangular=True), perm, q)


def is_upper_triangular(A, strict=False) -> bool:
    """No stored entry below the diagonal (strict: on or below) (_topological_sort.pyx:232-265)."""
    csr = _csr_int32(A)
    n = csr.shape[0]
    if n == 0:
        return True
    dev = require_cuda()
    d = _device_csr(csr)
    ws = torch.empty(256, dtype=torch.uint8, device=dev)
    res = ctypes.c_int32(1)
    ca = d.cstruct()
    _lib.check(_lib.load().rbg_is_upper_triangular_csr(ctypes.byref(ca), 1 if strict else 0, ctypes.byref(res),
                                                        ws.data_ptr(), ws.numel(), 0), "is_upper_triangular")
    return bool(res.value)
