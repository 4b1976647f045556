"""``extract_submatrix`` and ``merge_component_matrices`` of redblackgraph.sparse.csgraph
(_components.pyx:178-323) on the GPU: both are one ``rbg_csr_remap`` (rows and columns mapped
through index arrays, columns sorted)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ... import _lib
from ...device import csr_from_parts, require_cuda, to_device, to_host
from ...spgemm import DeviceCSR

__all__ = ["extract_submatrix", "merge_component_matrices"]


def _remap(csr, row_map: np.ndarray, col_map: np.ndarray, n_out: int):
    import scipy.sparse as sp
    dev = require_cuda()
    d = DeviceCSR.from_scipy(csr, dtype=np.int32)
    rm = to_device(np.ascontiguousarray(row_map, dtype=np.int32), dev)
    cm = to_device(np.ascontiguousarray(col_map if col_map.size else np.zeros(1), dtype=np.int32), dev)
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_csr_remap_workspace_bytes(n_out, d.nnz, ctypes.byref(nb)), "csr_remap")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    ip = torch.empty(n_out + 1, dtype=torch.int64, device=dev)
    cap = max(d.nnz, 1)
    oj = torch.empty(cap, dtype=torch.int32, device=dev)
    ox = torch.empty(cap, dtype=torch.int32, device=dev)
    nnz = ctypes.c_int64(0)
    ca = d.cstruct()
    _lib.check(L.rbg_csr_remap(ctypes.byref(ca), rm.data_ptr(), cm.data_ptr(), n_out, ip.data_ptr(), oj.data_ptr(),
                               ox.data_ptr(), cap, ws.data_ptr(), ws.numel(), ctypes.byref(nnz), 0), "csr_remap")
    m = int(nnz.value)
    return csr_from_parts(to_host(ox[:m]), to_host(oj[:m]), to_host(ip), (n_out, n_out))


def extract_submatrix(A, vertices):
    """The subgraph induced by ``vertices``, renumbered 0..k-1; returns (CSR, vertices as int32)."""
    import scipy.sparse as sp
    csr = A.tocsr() if sp.issparse(A) else sp.csr_matrix(A)
    n = csr.shape[0]
    verts = np.asarray(vertices, dtype=np.int32)
    k = verts.size
    old_to_new = np.full(max(n, 1), -1, np.int32)
    old_to_new[verts] = np.arange(k, dtype=np.int32)
    if n == 0 or k == 0:
        return sp.csr_matrix((k, k), dtype=np.int32), verts
    return _remap(csr, old_to_new[:n], old_to_new[:n], k), verts


def merge_component_matrices(components, n_total: int):
    """The full (n_total x n_total) CSR from (submatrix, new_to_old) pairs of extract_submatrix."""
    import scipy.sparse as sp
    comps = list(components)
    if not comps or n_total == 0:
        return sp.csr_matrix((n_total, n_total), dtype=np.int32)
    blocks = sp.block_diag([sp.csr_matrix(c[0]) for c in comps], format="csr")
    mapping = np.concatenate([np.asarray(c[1], dtype=np.int32) for c in comps])
    return _remap(sp.csr_matrix(blocks), mapping, mapping, int(n_total))
