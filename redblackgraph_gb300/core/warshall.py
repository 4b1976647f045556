"""``warshall`` -- the dense closure gufunc ``(m,m)->(m,m),()`` on the GPU.

Replaces the C gufunc registered at redblackgraph/core/src/redblackgraph/
redblackgraphmodule.c:583-597 (loops in warshall.c.in:51-135).  Each matrix of a stack is
closed with ``rbg_fw_dense``; W, the diameter and the exception (ValueError on a cycle,
OverflowError on an overflow -- the last error in loop order, as the reference reports) match
the reference.  One deliberate difference: for a stack of matrices the reference writes every
diameter into the first slot (its batch loop never advances the diameter pointer,
warshall.c.in:128); here each matrix gets its own diameter.
"""
from __future__ import annotations

import numpy as np

from .. import _lib
from ..dense import fw_dense, raise_for_core
from ..device import require_cuda, to_device, to_host

__all__ = ["warshall"]


def _check_input(A) -> np.ndarray:
    a = np.asarray(A)
    if a.dtype.kind not in "iu" or a.dtype.itemsize not in (1, 2, 4, 8):
        raise TypeError(f"ufunc 'warshall' not supported for the input types ({a.dtype})")
    if a.ndim < 2 or a.shape[-1] != a.shape[-2]:
        raise ValueError("warshall: core dimensions (m,m) must be square")
    return a


def warshall(A, out=None):
    """Return ``(W, diameter)``; W keeps the input's array subclass, diameter is int32."""
    a = _check_input(A)
    batch = a.shape[:-2]
    m = a.shape[-1]
    count = int(np.prod(batch)) if batch else 1
    flat = np.ascontiguousarray(a).reshape((count, m, m))
    W = np.empty_like(flat)
    diam = np.zeros(flat.shape[0], dtype=np.int32)
    last_err = None
    if m > 0 and flat.shape[0] > 0:
        dev = require_cuda()
        for b in range(flat.shape[0]):
            d = to_device(flat[b], dev)
            o, res = fw_dense(d, out=d, mode=0)
            if res.status != _lib.RBG_OK:
                last_err = res
                continue
            W[b] = to_host(o)
            diam[b] = res.diameter
    if last_err is not None:
        raise_for_core(last_err)
    W = W.reshape(a.shape)
    cls = type(A) if isinstance(A, np.ndarray) else np.ndarray
    W = W.view(cls)
    d = diam.reshape(batch) if batch else np.asarray(diam[0] if flat.shape[0] else 0, np.int32)
    if out is not None:
        o0, o1 = out if isinstance(out, tuple) else (out, None)
        if o0 is not None:
            o0[...] = W
            W = o0
        if o1 is not None:
            o1[...] = d
            d = o1
    return W, d
