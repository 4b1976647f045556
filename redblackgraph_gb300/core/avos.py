"""AVOS products on the GPU (the reference's redblackgraph/core/avos.py:1-17).

``einsum(..., avos=True)`` supports the four contractions ``rb.array @`` uses
(redblackgraph/core/redblack.py:14-38); ``avos_sum``/``avos_product`` evaluate the scalar
algebra of redblackgraph/core/src/redblackgraph/rbg_math.c.in:30-121 on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..device import default_workspace, require_cuda, stream_handle, to_device, to_host

__all__ = ["einsum", "avos_sum", "avos_product", "avos_matmul"]


def _common_dtype(a: np.ndarray, b: np.ndarray) -> np.dtype:
    dt = np.result_type(a.dtype, b.dtype)
    if dt.kind not in "iu" or dt.itemsize > 8:
        raise TypeError(f"AVOS product not supported for the input types ({a.dtype}, {b.dtype})")
    return dt


def matmul_device(a, b, out=None, stream=None):
    """C = a (x) b on device tensors (2-D, same integer dtype)."""
    from ..device import numpy_dtype
    m, q = a.shape
    q2, p = b.shape
    if q != q2:
        raise ValueError("matmul: inner dimensions differ")
    import torch
    a = a.contiguous()
    b = b.contiguous()
    if out is None:
        out = torch.empty((m, p), dtype=a.dtype, device=a.device)
    L = _lib.load()
    code = _lib.dtype_code(numpy_dtype(a.dtype))
    nb = ctypes.c_int64(0)
    _lib.check(L.rbg_avos_matmul_workspace_bytes(code, m, q, p, ctypes.byref(nb)), "avos_matmul")
    ws = default_workspace().get(nb.value, a.device)
    flags = ctypes.c_uint32(0)
    rc = L.rbg_avos_matmul(code, m, q, p, a.data_ptr(), q, b.data_ptr(), p, out.data_ptr(), p,
                           ws.data_ptr(), ws.numel(), ctypes.byref(flags), stream_handle(stream))
    return out, rc, flags.value


def avos_matmul(a: np.ndarray, b: np.ndarray):
    """``a @ b`` for 1-D/2-D host operands, computed on the GPU."""
    a = np.asarray(a)
    b = np.asarray(b)
    dt = _common_dtype(a, b)
    A = a.astype(dt, copy=False)
    B = b.astype(dt, copy=False)
    av, bv = A.ndim == 1, B.ndim == 1
    A2 = A.reshape(1, -1) if av else A
    B2 = B.reshape(-1, 1) if bv else B
    if A2.shape[1] != B2.shape[0]:
        raise ValueError(f"operands could not be broadcast together with shapes {a.shape} {b.shape}")
    dev = require_cuda()
    m, p = A2.shape[0], B2.shape[1]
    if A2.shape[1] == 0 or m == 0 or p == 0:
        C = np.zeros((m, p), dt)
    else:
        out, rc, flags = matmul_device(to_device(A2, dev), to_device(B2, dev))
        if rc == _lib.RBG_ERR_OVERFLOW:
            raise OverflowError("Avos product results in an overflow.")
        _lib.check(rc, "avos_matmul")
        C = to_host(out)
    if av and bv:
        return C.reshape(())[()]
    if av:
        return C.reshape(p)
    if bv:
        return C.reshape(m)
    return C


def einsum(*operands, **kwargs):
    avos = kwargs.pop("avos", False)
    if not avos:
        raise ValueError("Avos should be specified in all cases.")
    spec, a, b = operands
    if spec in ("ij,jk", "i,i", "i,...ij", "...i,i"):
        return avos_matmul(a, b)
    raise ValueError(f"unsupported AVOS contraction {spec!r}")


def avos_sum(lhs: int, rhs: int, dtype=np.int64) -> int:
    from ..elementwise import avos_sum_array
    return int(avos_sum_array(np.array([lhs], dtype), np.array([rhs], dtype))[0])


def avos_product(lhs: int, rhs: int, dtype=np.int64) -> int:
    from ..elementwise import avos_product_array
    r = avos_product_array(np.array([lhs]).astype(dtype), np.array([rhs]).astype(dtype))
    return int(r[0])
