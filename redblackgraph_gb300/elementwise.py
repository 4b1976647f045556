"""Element-wise AVOS sum / product over arrays, on the GPU (``rbg_avos_elementwise``)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .device import default_workspace, require_cuda, stream_handle, to_device, to_host


def _run(op: int, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x)
    y = np.ascontiguousarray(y, dtype=x.dtype)
    if x.shape != y.shape:
        raise ValueError("operands must have the same shape")
    dev = require_cuda()
    dx, dy = to_device(x.reshape(-1), dev), to_device(y.reshape(-1), dev)
    dz = dx.clone()
    ws = default_workspace().get(256, dev)
    flags = ctypes.c_uint32(0)
    rc = _lib.load().rbg_avos_elementwise(op, _lib.dtype_code(x.dtype), x.size, dx.data_ptr(),
                                          dy.data_ptr(), dz.data_ptr(), ws.data_ptr(), ws.numel(),
                                          ctypes.byref(flags), stream_handle())
    if rc == _lib.RBG_ERR_OVERFLOW:
        raise OverflowError("Avos product results in an overflow.")
    _lib.check(rc, "avos_elementwise")
    z = to_host(dz).reshape(x.shape)
    if op == 1 and x.dtype.kind == "i":
        z = z.view(np.dtype(f"u{x.dtype.itemsize}"))
    return z


def avos_sum_array(x, y):
    return _run(0, np.asarray(x), np.asarray(y))


def avos_product_array(x, y):
    return _run(1, np.asarray(x), np.asarray(y))
