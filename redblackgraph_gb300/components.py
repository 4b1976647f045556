"""Component-wise closure on the GPU, at the device-tensor level.

When every component is numbered in a topological order and clean, the closure is taken
straight from the CSR graph (``dag_component_closure``: the DAG recurrence per component, the
Floyd-Warshall diameter from each cell's first value).  Otherwise:

The graph (device CSR: int64 row pointers, int32 column indices, int32 values) is split into
connected components by ``rbg_cc_label``, each component is scattered into its own dense block
of one flat buffer (``rbg_cc_densify``), all blocks are closed by one ``rbg_fw_batch`` call in
the Cython semantics, and the closed blocks are compacted back into one CSR matrix with global
indices (``rbg_cc_compact_scan`` of the row counts the closure recorded, or
``rbg_cc_compact_count``, then ``rbg_cc_compact_fill``).  Mirrors component_wise_closure,
redblackgraph/sparse/csgraph/transitive_closure.py:85-195, whose per-component loop this batch
replaces.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import stream_handle
from .dense import fw_batch, raise_for_cython


@dataclass
class Components:
    """Connected components of an n-vertex graph, on the device."""
    n: int
    count: int
    label: torch.Tensor          # int32 [n]: component of each vertex (numbered by least vertex)
    sorted_vertex: torch.Tensor  # int32 [n]: vertices grouped by component, ascending
    local: torch.Tensor          # int32 [n]: index of each vertex inside its component
    start: torch.Tensor          # int64 [n + 1]: component c is sorted_vertex[start[c]:start[c+1]]
    workspace: torch.Tensor      # uint8 scratch shared by the rbg_cc_* calls
    sizes: np.ndarray            # int64 [count] on the host


@dataclass
class DenseBlocks:
    flat: torch.Tensor           # int32: every component's dense block, one after another
    sizes: np.ndarray            # int64 [count]
    offsets: np.ndarray          # int64 [count] element offsets into flat
    dense_off: torch.Tensor      # the same offsets on the device


def label_components(indptr: torch.Tensor, indices: torch.Tensor, n: int, stream=None) -> Components:
    """Connected components with edges taken in both directions (_components.pyx:86-177)."""
    dev = indptr.device
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_cc_workspace_bytes(n, ctypes.byref(nb)), "cc_workspace_bytes")
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
    label = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    sv = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    local = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    start = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    nc = ctypes.c_int64(0)
    idx_ptr = indices.data_ptr() if indices.numel() else indptr.data_ptr()
    _lib.check(L.rbg_cc_label(n, indptr.data_ptr(), idx_ptr, ws.data_ptr(), ws.numel(), label.data_ptr(),
                              sv.data_ptr(), local.data_ptr(), start.data_ptr(), ctypes.byref(nc),
                              stream_handle(stream)), "cc_label")
    count = nc.value
    sizes = np.diff(start[:count + 1].cpu().numpy()) if count else np.zeros(0, np.int64)
    return Components(n, count, label, sv, local, start, ws, sizes.astype(np.int64))


def densify(indptr, indices, data, comps: Components, stream=None) -> DenseBlocks:
    """Scatter the stored values into one dense block per component (zeros elsewhere)."""
    sizes = comps.sizes
    offsets = np.zeros_like(sizes)
    if sizes.size > 1:
        offsets[1:] = np.cumsum(sizes[:-1] * sizes[:-1])
    total = int((sizes * sizes).sum())
    dev = indptr.device
    flat = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    dense_off = torch.from_numpy(offsets if offsets.size else np.zeros(1, np.int64)).to(dev)
    L = _lib.load()
    ip = indptr.data_ptr()
    _lib.check(L.rbg_cc_densify(_lib.dtype_code(np.int32), comps.n, ip, indices.data_ptr() if indices.numel() else ip,
                                data.data_ptr() if data.numel() else ip, comps.label.data_ptr(),
                                comps.local.data_ptr(), comps.start.data_ptr(), dense_off.data_ptr(),
                                flat.data_ptr(), total, stream_handle(stream)), "cc_densify")
    return DenseBlocks(flat, sizes, offsets, dense_off)


def chunk_mask_buffer(comps: Components, blocks: DenseBlocks) -> torch.Tensor:
    """Device words for the per-row 32-column chunk masks of the closed blocks."""
    mw = ctypes.c_int64(0)
    _lib.check(_lib.load().rbg_cc_chunk_mask_words(comps.n, comps.count, blocks.flat.numel(), ctypes.byref(mw)),
               "cc_chunk_mask_words")
    return torch.empty(max(mw.value, 1), dtype=torch.int64, device=blocks.flat.device)


def compact(comps: Components, blocks: DenseBlocks, want_max: bool = False, stream=None,
            counted: tuple | None = None):
    """Merge the closed blocks into one CSR matrix (_components.pyx:254-324).

    ``counted = (row_count, mask, comp_max)``: the per-row statistics the closure recorded
    (rbg_fw_batch_rows); the blocks are then read once, by the fill.  Returns
    ``(indptr int64, indices int32, data int32, comp_max or None)``."""
    dev = blocks.flat.device
    L = _lib.load()
    n, k = comps.n, comps.count
    nnz = ctypes.c_int64(0)
    sh = stream_handle(stream)
    args = (comps.label.data_ptr(), comps.local.data_ptr(), comps.start.data_ptr(),
            blocks.dense_off.data_ptr(), blocks.flat.data_ptr())
    if counted is not None:
        row_count, mask, cmax = counted
        _lib.check(L.rbg_cc_compact_scan(n, row_count.data_ptr(), comps.workspace.data_ptr(),
                                         comps.workspace.numel(), ctypes.byref(nnz), sh), "cc_compact_scan")
    else:
        cmax = torch.empty(max(k, 1), dtype=torch.int32, device=dev) if want_max else None
        mask = chunk_mask_buffer(comps, blocks)     # which 32-column chunks hold values
        _lib.check(L.rbg_cc_compact_count(n, k, *args, comps.workspace.data_ptr(), comps.workspace.numel(),
                                          ctypes.byref(nnz), cmax.data_ptr() if cmax is not None else None,
                                          mask.data_ptr(), sh),
                   "cc_compact_count")
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
    data = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_cc_compact_fill(n, *args, comps.sorted_vertex.data_ptr(), comps.workspace.data_ptr(),
                                     indptr.data_ptr(), indices.data_ptr(), data.data_ptr(), mask.data_ptr(), sh),
               "cc_compact_fill")
    return indptr, indices[:nnz.value], data[:nnz.value], cmax


def component_methods(sizes: np.ndarray, count: int, method: str, densify_threshold: int) -> np.ndarray:
    """True where a component takes the Floyd-Warshall diameter, False for the 'D' one
    (transitive_closure.py:151-187: a single component takes "FW" only when asked for; with
    "auto" components up to ``densify_threshold`` vertices take "FW"; any other method string
    runs the 'D' branch)."""
    if count == 1:
        return np.array([method == "FW"])
    if method == "auto":
        return sizes <= densify_threshold
    return np.full(sizes.shape, method == "FW")


def _msb(v: int) -> int:
    return v.bit_length() - 1 if v > 1 else 0


DAG_MAX_N = 8192          # rows of a component the DAG path takes (include/rbg_gb300.h)
_UNCLEAN, _BELOW, _ABOVE = 1, 2, 4


def dag_component_closure(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor, n: int,
                          comps: Components, method: str, densify_threshold: int, stream=None):
    """Component-wise closure straight from the CSR graph when every component is numbered in a
    topological order (entries all below, or all above, the diagonal), clean and at most 8192
    vertices: closure rows by the DAG recurrence, Floyd-Warshall diameters from each cell's first
    value, the diagonal put back (rbg_cc_dag_*).  Returns ``(indptr, indices, data, diameter)``,
    or None when some component needs the dense path (or a product may reach the top bit)."""
    from .dag import RowTooWide, dag_closure_device
    from .spgemm import DeviceCSR
    k = comps.count
    if k == 0 or int(comps.sizes.max()) > DAG_MAX_N:
        return None
    L = _lib.load()
    dev = indptr.device
    sh = stream_handle(stream)
    ws = comps.workspace
    ip = indptr.data_ptr()
    ij = indices.data_ptr() if indices.numel() else ip
    iv = data.data_ptr() if data.numel() else ip
    flags = torch.empty(k, dtype=torch.int32, device=dev)
    diag = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    eptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    ne = ctypes.c_int64(0)
    _lib.check(L.rbg_cc_dag_classify(n, ip, ij, iv, comps.sorted_vertex.data_ptr(), comps.start.data_ptr(), k,
                                     ws.data_ptr(), ws.numel(), flags.data_ptr(), diag.data_ptr(), eptr.data_ptr(),
                                     ctypes.byref(ne), sh), "cc_dag_classify")
    f = flags.cpu().numpy()
    if ((f & _UNCLEAN) != 0).any() or (((f & _BELOW) != 0) & ((f & _ABOVE) != 0)).any():
        return None
    kind = torch.from_numpy(np.where(f & _ABOVE, 2, 1).astype(np.int32)).to(dev)
    ecol = torch.empty(max(ne.value, 1), dtype=torch.int32, device=dev)
    evals = torch.empty(max(ne.value, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_cc_dag_edges(n, ip, ij, iv, eptr.data_ptr(), ecol.data_ptr(), evals.data_ptr(), sh),
               "cc_dag_edges")
    E = DeviceCSR(eptr, ecol[:ne.value], evals[:ne.value], (n, n))
    try:
        C, _, _ = dag_closure_device(E, stream, gather=False)    # the row pool, read in place
    except RowTooWide:
        return None
    top = torch.empty(k, dtype=torch.int32, device=dev)
    first = torch.empty(k, dtype=torch.int32, device=dev)
    cmax = torch.empty(k, dtype=torch.int32, device=dev)
    ec = E.cstruct()
    pool = (C.row_off.data_ptr(), C.row_len.data_ptr(), C.cols.data_ptr(), C.vals.data_ptr())
    _lib.check(L.rbg_cc_dag_stats(n, k, comps.label.data_ptr(), comps.local.data_ptr(), comps.start.data_ptr(),
                                  comps.sorted_vertex.data_ptr(), kind.data_ptr(), ctypes.byref(ec), *pool,
                                  diag.data_ptr(), top.data_ptr(), first.data_ptr(), cmax.data_ptr(), sh),
               "cc_dag_stats")
    st = torch.stack([top, first, cmax]).cpu().numpy()
    if (st[0] >= 31).any():
        return None
    oi = torch.empty(n + 1, dtype=torch.int64, device=dev)
    nnz = ctypes.c_int64(0)
    _lib.check(L.rbg_cc_dag_merge_count(n, C.row_len.data_ptr(), diag.data_ptr(), ws.data_ptr(), ws.numel(),
                                        oi.data_ptr(), ctypes.byref(nnz), sh), "cc_dag_merge_count")
    oj = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
    ov = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
    _lib.check(L.rbg_cc_dag_merge_fill(n, *pool, diag.data_ptr(), oi.data_ptr(), oj.data_ptr(), ov.data_ptr(), sh),
               "cc_dag_merge_fill")
    fw = component_methods(comps.sizes, k, method, densify_threshold)
    diameter = 0
    if fw.any():
        diameter = max(0, int(st[1][fw].max()))
    if (~fw).any():
        diameter = max(diameter, _msb(int(st[2][~fw].max())))
    return oi, oj[:nnz.value], ov[:nnz.value], diameter


def component_closure_device(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor, n: int,
                             method: str = "auto", densify_threshold: int = 500, stream=None):
    """Close every component of the device CSR graph.

    Returns ``(indptr, indices, data, diameter, comps)``; raises CycleError for the first
    component (by number) that holds a cycle, as the reference's per-component loop does.
    """
    comps = label_components(indptr, indices, n, stream)
    got = dag_component_closure(indptr, indices, data, n, comps, method, densify_threshold, stream)
    if got is not None:
        return (*got, comps)
    blocks = densify(indptr, indices, data, comps, stream)
    fw = component_methods(comps.sizes, comps.count, method, densify_threshold)
    # the closure's finalization counts every row while it writes it (one read of the blocks less)
    dev = blocks.flat.device
    row_count = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    mask = chunk_mask_buffer(comps, blocks)
    cmax = None if fw.all() else torch.zeros(max(comps.count, 1), dtype=torch.int32, device=dev)
    stats = _lib.RbgRowStats(comps.start.data_ptr(), comps.sorted_vertex.data_ptr(), row_count.data_ptr(),
                             mask.data_ptr(), cmax.data_ptr() if cmax is not None else None)
    _, res = fw_batch(blocks.flat, blocks.sizes, blocks.offsets, out=blocks.flat,
                      mode=_lib.MODE_CYTHON | _lib.MODE_GRAPH | _lib.MODE_AUTOTUNE, stream=stream,
                      as_array=True, row_stats=stats)
    bad = np.flatnonzero(res["status"] != _lib.RBG_OK)
    if bad.size:                                     # the first component (by number) raises
        r = _lib.RbgResult()
        ctypes.memmove(ctypes.addressof(r), res[bad[0]:bad[0] + 1].tobytes(), ctypes.sizeof(r))
        raise_for_cython(r)
    # components closed on another path have no recorded statistics: count every row again
    recorded = (res["path"] == _lib.PATH_BLOCKED32) | (res["path"] == _lib.PATH_DAG)
    counted = (row_count, mask, cmax) if bool(recorded.all()) else None
    oi, oj, ov, cmax = compact(comps, blocks, want_max=not bool(fw.all()), stream=stream, counted=counted)
    diameter = 0
    if fw.any():
        diameter = int(res["diameter"][fw].max())
    if cmax is not None:
        mx = cmax[:comps.count].cpu().numpy()
        diameter = max(diameter, _msb(int(mx[~fw].max())))
    return oi, oj, ov, diameter, comps
