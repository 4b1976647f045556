"""Relational composition on the GPU: the closure of a closed graph after adding one vertex or
one edge, without recomputing the closure (``rbg_vertex_compose`` / ``rbg_edge_compose``).

Mirrors the C core gufuncs (redblackgraph/core/src/redblackgraph/relational_composition.c.in:
72-262, reached through redblackgraph/core/redblack.py:52-130) and the Cython functions
(redblackgraph/sparse/csgraph/_relational_composition.pyx:10-113): same arguments, results and
exceptions.  The device functions work on resident closures and can update one in place, which
is what a serving loop uses to apply a mutation: only the rows that reach the new vertex (or
the edge's source) times the columns it reaches are touched.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import default_workspace, numpy_dtype, require_cuda, stream_handle, to_device, to_host

__all__ = ["vertex_compose_device", "edge_compose_device", "raise_for_compose", "vertex_compose_host",
           "edge_compose_host"]


def _workspace(code: int, n: int, device):
    L = _lib.load()
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_compose_workspace_bytes(code, n, ctypes.byref(nb)), "compose")
    return default_workspace().get(max(nb.value, 256), device)


def vertex_compose_device(R: torch.Tensor, u: torch.Tensor, v: torch.Tensor, color: int, out=None,
                          mode: int = 0, stream=None, n: int | None = None):
    """R_lambda for the closed device matrix R (its top-left n x n block; n defaults to R's
    size), new vertex row u and column v (device vectors of n) and colour ``color``.  ``out``
    is an (n+1) x (n+1) device matrix, allocated when None; ``out is R`` (a buffer of at least
    n + 1 rows and columns) updates in place.  Returns ``(out, RbgComposeResult)``."""
    if R.ndim != 2 or not R.is_cuda:
        raise ValueError("vertex_compose_device takes a 2-D CUDA tensor")
    n = R.shape[0] if n is None else int(n)
    if out is None:
        out = torch.empty((n + 1, n + 1), dtype=R.dtype, device=R.device)
    if out.shape[0] < n + 1 or out.shape[1] < n + 1 or out.dtype != R.dtype:
        raise ValueError("out must be at least (n+1) x (n+1) of R's dtype")
    if u.dtype != R.dtype or v.dtype != R.dtype or u.numel() < n or v.numel() < n:
        raise ValueError("u and v must be n values of R's dtype")
    code = _lib.dtype_code(numpy_dtype(R.dtype))
    ws = _workspace(code, n, R.device)
    res = _lib.RbgComposeResult()
    L = _lib.load()
    rc = L.rbg_vertex_compose(code, n, R.data_ptr(), R.stride(0), u.data_ptr(), v.data_ptr(), int(color),
                              out.data_ptr(), out.stride(0), mode, ws.data_ptr(), ws.numel(), ctypes.byref(res),
                              stream_handle(stream))
    _lib.check(rc, "vertex_compose")
    return out, res


def edge_compose_device(R: torch.Tensor, alpha: int, beta: int, relationship: int, out=None, mode: int = 0,
                        stream=None):
    """R' for the closed device matrix R with the edge alpha -> beta of value ``relationship``;
    ``out is R`` updates in place.  Returns ``(out, RbgComposeResult)``."""
    if R.ndim != 2 or R.shape[0] != R.shape[1] or not R.is_cuda:
        raise ValueError("edge_compose_device takes a square CUDA tensor")
    n = R.shape[0]
    if out is None:
        out = torch.empty_like(R)
    code = _lib.dtype_code(numpy_dtype(R.dtype))
    ws = _workspace(code, n, R.device)
    res = _lib.RbgComposeResult()
    L = _lib.load()
    rc = L.rbg_edge_compose(code, n, R.data_ptr(), R.stride(0), int(alpha), int(beta), int(relationship),
                            out.data_ptr(), out.stride(0), mode, ws.data_ptr(), ws.numel(), ctypes.byref(res),
                            stream_handle(stream))
    _lib.check(rc, "edge_compose")
    return out, res


def _as_type(x: int, dtype) -> int:
    """The value bits ``x`` (widened to 64 bits) read in ``dtype``."""
    return int(np.array(x, dtype=np.int64).astype(np.uint64).astype(dtype))


def raise_for_compose(res: _lib.RbgComposeResult, dtype) -> None:
    """Raise what the C core raises (relational_composition.c.in:221-227, rbg_math.c.in:103-118)."""
    if res.status == _lib.RBG_OK:
        return
    if res.status == _lib.RBG_ERR_CYCLE:
        raise ValueError(f"Relational composition would result in a cycle. Idx: {res.i}, "
                         f"u_i: {_as_type(res.lhs, dtype)}, v_i: {_as_type(res.rhs, dtype)}")
    if res.status == _lib.RBG_ERR_OVERFLOW:
        a, b = _as_type(res.lhs, dtype), _as_type(res.rhs, dtype)
        if res.event & _lib.EV_HANG:
            raise OverflowError(f"Avos product of {a} and {b} has a negative signed operand; its bit length "
                                "is undefined (the reference does not return here)")
        if res.event & _lib.EV_OVF_ONES:
            raise OverflowError(f"Avos product of {a} and {b}, results in an overflow. Result of avos "
                                "product collides with 'red' 1 (-1).")
        bits = np.dtype(dtype).itemsize * 8
        need = _msb(a, dtype) + _msb(b, dtype) + 1
        raise OverflowError(f"Avos product of {a} and {b}, results in an overflow. (Result size would "
                            f"require {need} bits; Type provides {bits} bits)")
    raise RuntimeError(f"relational composition failed with status {res.status}")


def _msb(x: int, dtype) -> int:
    u = int(np.array(x, dtype=dtype).astype(np.uint64)) & ((1 << (np.dtype(dtype).itemsize * 8)) - 1)
    return max(u.bit_length() - 1, 0)


def vertex_compose_host(u, R, v, color, cython: bool = False) -> np.ndarray:
    """Vertex composition of host arrays through the GPU (H2D, one composition, D2H)."""
    R = np.ascontiguousarray(R)
    dev = require_cuda()
    n = R.shape[0]
    dR = to_device(R, dev)
    du = to_device(np.ascontiguousarray(np.asarray(u).reshape(-1)[:n], dtype=R.dtype), dev)
    dv = to_device(np.ascontiguousarray(np.asarray(v).reshape(-1)[:n], dtype=R.dtype), dev)
    out, res = vertex_compose_device(dR, du, dv, color, mode=_lib.MODE_CYTHON if cython else 0)
    raise_for_compose(res, R.dtype)
    return to_host(out)


def edge_compose_host(R, alpha, beta, relationship, cython: bool = False) -> np.ndarray:
    """Edge composition of a host array through the GPU."""
    R = np.ascontiguousarray(R)
    dev = require_cuda()
    dR = to_device(R, dev)
    out, res = edge_compose_device(dR, alpha, beta, relationship, mode=_lib.MODE_CYTHON if cython else 0)
    raise_for_compose(res, R.dtype)
    return to_host(out)
