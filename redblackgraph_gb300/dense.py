"""Dense AVOS closure on the GPU, at the tensor level.

``fw_dense`` runs ``rbg_fw_dense`` (include/rbg_gb300.h) on a square device tensor.  The
Python entry points that mirror the reference (``core.warshall``, ``array.transitive_closure``,
``sparse.csgraph.floyd_warshall``) are thin wrappers over it.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import default_workspace, require_cuda, stream_handle, numpy_dtype, to_device, to_host


class CycleError(ValueError):
    """Raised by the csgraph closure when a vertex reaches itself.

    Mirrors redblackgraph/sparse/csgraph/cycleerror.py:1-6 (a ValueError carrying
    ``vertex``)."""

    def __init__(self, *args, **kwargs):
        super().__init__(args, kwargs)
        self.vertex = kwargs.get("vertex")


def fw_dense(a: torch.Tensor, out: torch.Tensor | None = None, mode: int = 0,
             stream: torch.cuda.Stream | None = None) -> tuple[torch.Tensor, _lib.RbgResult]:
    """Close the (n, n) device tensor ``a`` into ``out`` (allocated when None; may be ``a``).

    Returns ``(out, result)``; ``result.status`` is the reference's error, not raised here.
    """
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError("expected a square matrix")
    if not a.is_cuda:
        raise ValueError("fw_dense takes a CUDA tensor")
    a = a.contiguous()
    n = a.shape[0]
    if out is None:
        out = torch.empty_like(a)
    code = _lib.dtype_code(numpy_dtype(a.dtype))
    L = _lib.load()
    nbytes = ctypes.c_int64(0)
    _lib.check(L.rbg_fw_dense_workspace_bytes(code, n, mode, ctypes.byref(nbytes)), "fw_dense")
    ws = default_workspace().get(nbytes.value, a.device)
    res = _lib.RbgResult()
    rc = L.rbg_fw_dense(code, n, a.data_ptr(), n, out.data_ptr(), out.stride(0), mode,
                        ws.data_ptr(), ws.numel(), ctypes.byref(res), stream_handle(stream))
    _lib.check(rc, "fw_dense")
    return out, res


def raise_for_core(res: _lib.RbgResult) -> None:
    """Raise what the C core gufunc raises (warshall.c.in:82-86, rbg_math.c.in:103-118)."""
    if res.status == _lib.RBG_OK:
        return
    if res.status == _lib.RBG_ERR_OVERFLOW:
        if res.flags & _lib.EV_HANG:
            raise OverflowError(
                f"Avos product at A({res.i},{res.k}) x A({res.k},{res.j}) has a negative signed "
                "operand; its bit length is undefined (the reference does not return here)")
        raise OverflowError(
            f"Avos product at A({res.i},{res.k}) x A({res.k},{res.j}) results in an overflow.")
    if res.status == _lib.RBG_ERR_CYCLE:
        raise ValueError(
            f"Error: cycle detected! Vertex {res.i} has a path to itself. "
            f"A({res.i},{res.k}), A({res.k},{res.j})")
    raise RuntimeError(f"closure failed with status {res.status}")


def raise_for_cython(res: _lib.RbgResult) -> None:
    """Raise what _floyd_warshall_avos raises (_shortest_path.pyx:376,386)."""
    if res.status == _lib.RBG_OK:
        return
    if res.status == _lib.RBG_ERR_CYCLE:
        raise CycleError(f"Error: cycle detected! Vertex {res.i} has a path to itself. "
                         f"A({res.i},{res.k}), A({res.k},{res.j})", vertex=int(res.i))
    raise RuntimeError(f"closure failed with status {res.status}")


def warshall_host(A: np.ndarray, mode: int = 0) -> tuple[np.ndarray, int, _lib.RbgResult]:
    """Close one host matrix on the GPU: H2D, ``rbg_fw_dense``, D2H."""
    A = np.ascontiguousarray(A)
    dev = require_cuda()
    if A.shape[0] == 0:
        return A.copy(), 0, _lib.RbgResult()
    d = to_device(A, dev)
    out, res = fw_dense(d, out=d, mode=mode)
    return to_host(out), int(res.diameter), res


def fw_batch(buf: torch.Tensor, sizes, offsets, out: torch.Tensor | None = None, mode: int = 0,
             stream: torch.cuda.Stream | None = None, as_array: bool = False,
             row_stats: "_lib.RbgRowStats | None" = None) -> tuple[torch.Tensor, list]:
    """Close many matrices packed in one flat device tensor ``buf``.

    Matrix i is ``sizes[i] x sizes[i]`` at element offset ``offsets[i]``.  Returns
    ``(out, results)`` with one ``RbgResult`` per matrix, or with ``as_array`` a numpy
    structured array of ``_lib.RESULT_DTYPE`` records (no per-matrix Python objects).
    With ``row_stats`` (int32 only) the finalization also records the per-row statistics of
    ``rbg_fw_batch_rows`` for every matrix closed by the 32-bit blocked pass.
    """
    import numpy as np
    if not buf.is_cuda or buf.ndim != 1:
        raise ValueError("fw_batch takes a flat CUDA tensor")
    sizes = np.ascontiguousarray(sizes, dtype=np.int64)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    if sizes.shape != offsets.shape:
        raise ValueError("sizes and offsets differ in length")
    if sizes.size and int((offsets + sizes * sizes).max()) > buf.numel():
        raise ValueError("a matrix extends past the end of the buffer")
    if out is None:
        out = torch.empty_like(buf)
    count = int(sizes.size)
    code = _lib.dtype_code(numpy_dtype(buf.dtype))
    L = _lib.load()
    nbytes = ctypes.c_int64(0)
    _lib.check(L.rbg_fw_batch_workspace_bytes(code, count, sizes.ctypes.data, mode,
                                              ctypes.byref(nbytes)), "fw_batch")
    ws = default_workspace().get(nbytes.value, buf.device)
    results = (_lib.RbgResult * max(count, 1))()
    if row_stats is not None:
        rc = L.rbg_fw_batch_rows(code, count, sizes.ctypes.data, offsets.ctypes.data, buf.data_ptr(),
                                 out.data_ptr(), mode, ws.data_ptr(), ws.numel(), ctypes.byref(row_stats),
                                 results, stream_handle(stream))
    else:
        rc = L.rbg_fw_batch(code, count, sizes.ctypes.data, offsets.ctypes.data, buf.data_ptr(),
                            out.data_ptr(), mode, ws.data_ptr(), ws.numel(), results,
                            stream_handle(stream))
    _lib.check(rc, "fw_batch")
    if as_array:
        return out, np.frombuffer(results, dtype=_lib.RESULT_DTYPE, count=count).copy()
    return out, [results[i] for i in range(count)]


def pack(mats):
    """Pack host matrices into one flat array; returns (flat, sizes, offsets)."""
    import numpy as np
    sizes = np.array([m.shape[0] for m in mats], dtype=np.int64)
    offsets = np.zeros_like(sizes)
    if len(mats) > 1:
        offsets[1:] = np.cumsum(sizes[:-1] * sizes[:-1])
    total = int((sizes * sizes).sum())
    dt = mats[0].dtype if mats else np.int32
    flat = np.empty(total, dtype=dt)
    for m, o in zip(mats, offsets):
        flat[o:o + m.size] = np.ascontiguousarray(m).reshape(-1)
    return flat, sizes, offsets
