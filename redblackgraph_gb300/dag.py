"""Closure of a DAG by topological levels on the GPU (``rbg_dag_closure`` / ``rbg_dag_gather``).

The reference's sparse DAG closure (redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:
168-351) builds every vertex's row from its parents' closed rows; here all rows of one
topological level are built at once on the device.  The closure rows land in a row pool whose
size is not known in advance (each row reserves its bound: stored entries plus its parents' row
lengths): the pool starts at a multiple of nnz(A) and grows (the call is repeated) when the
library reports it too small.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import stream_handle
from .spgemm import DeviceCSR


class RowTooWide(RuntimeError):
    """A closure row has more distinct columns than the level kernels hold (8192)."""


@dataclass
class DagRows:
    """The closure's rows as rbg_dag_closure leaves them in its row pool: row v is
    cols[row_off[v]:row_off[v] + row_len[v]] (columns ascending) with its values in vals."""
    cols: torch.Tensor
    vals: torch.Tensor
    row_off: torch.Tensor      # int64 [n]
    row_len: torch.Tensor      # int32 [n]
    nnz: int


def dag_closure_device(A: DeviceCSR, stream=None, pool_factor: int = 16, gather: bool = True):
    """Closure of the DAG ``A`` (int32 values).  Returns ``(C, max_abs, levels)``: the closure as
    a DeviceCSR (int64 row pointers, int32 indices and values, rows sorted) -- or, with
    ``gather=False``, as the row pool itself (``DagRows``) -- the largest magnitude among A's
    entries and all candidates (the reference's diameter source) and the number of topological
    levels.  Raises CycleError on a cycle and RowTooWide for rows past 8192 columns."""
    from .dense import CycleError
    if A.data.dtype != torch.int32:
        raise TypeError("the DAG closure takes int32 values")
    n = A.shape[0]
    dev = A.indptr.device
    if n == 0:
        z = torch.zeros(1, dtype=torch.int64, device=dev)
        return DeviceCSR(z, torch.zeros(0, dtype=torch.int32, device=dev),
                         torch.zeros(0, dtype=torch.int32, device=dev), (0, 0)), 0, 0
    L = _lib.load()
    sh = stream_handle(stream)
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_dag_workspace_bytes(n, A.nnz, ctypes.byref(nb)), "dag_workspace")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    row_off = torch.empty(n, dtype=torch.int64, device=dev)
    row_len = torch.empty(n, dtype=torch.int32, device=dev)
    cap = max(pool_factor * A.nnz + n, 1024)
    ca = A.cstruct()
    while True:
        cols = torch.empty(cap, dtype=torch.int32, device=dev)
        vals = torch.empty(cap, dtype=torch.int32, device=dev)
        nnz, mx, lv = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        rc = L.rbg_dag_closure(ctypes.byref(ca), ws.data_ptr(), ws.numel(), cols.data_ptr(), vals.data_ptr(), cap,
                               row_off.data_ptr(), row_len.data_ptr(), ctypes.byref(nnz), ctypes.byref(mx),
                               ctypes.byref(lv), sh)
        if rc == _lib.RBG_ERR_CYCLE:
            raise CycleError("transitive_closure_dag_sparse requires a DAG (no cycles)", vertex=-1)
        if rc == _lib.RBG_ERR_CAPACITY:
            if nnz.value < 0:
                raise RowTooWide("a closure row has more than 8192 distinct columns")
            cap = int(nnz.value)
            del cols, vals
            continue
        _lib.check(rc, "dag_closure")
        break
    total = int(nnz.value)
    if not gather:
        return DagRows(cols, vals, row_off, row_len, total), int(mx.value), int(lv.value)
    gb = ctypes.c_int64(0)
    _lib.check(L.rbg_dag_gather_workspace_bytes(n, ctypes.byref(gb)), "dag_gather")
    gws = torch.empty(max(gb.value, 256), dtype=torch.uint8, device=dev)
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    data = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_dag_gather(n, cols.data_ptr(), vals.data_ptr(), row_off.data_ptr(), row_len.data_ptr(),
                                gws.data_ptr(), gws.numel(), indptr.data_ptr(), indices.data_ptr(),
                                data.data_ptr(), sh), "dag_gather")
    return DeviceCSR(indptr, indices[:total], data[:total], (n, n)), int(mx.value), int(lv.value)
