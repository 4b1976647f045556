"""Dense red/black matrices: ``array`` with AVOS ``@`` and ``transitive_closure``.

Mirrors redblackgraph/core/redblack.py:11-129 -- same class names, operators, results and
exceptions -- but every product and closure runs on the GPU through librbg_gb300.so
(``rbg_avos_matmul``, ``rbg_fw_dense``).
"""
from __future__ import annotations

import numpy as np
from numpy import ndarray, asarray

from ..types import TransitiveClosure
from .avos import avos_matmul
from .warshall import warshall

__all__ = ["array", "transitive_closure", "warshall"]


class _Avos(ndarray):
    """AVOS ``@`` for 1-D/2-D operands (redblack.py:14-38 einsum forms)."""

    def __matmul__(self, other):
        other = np.asarray(other)
        if self.ndim in (1, 2) and other.ndim in (1, 2):
            return avos_matmul(np.asarray(self), other)
        raise ValueError(f"Unexpected dimensionality. self: {self.ndim}, other: {other.ndim}")

    def __rmatmul__(self, other):
        other = np.asarray(other)
        if self.ndim in (1, 2) and other.ndim in (1, 2):
            return avos_matmul(other, np.asarray(self))
        raise ValueError(f"Unexpected dimensionality. self: {self.ndim}, other: {other.ndim}")

    def cardinality(self):
        trace = np.trace(self)
        m = self.shape[0]
        c_black = int((m + trace) / 2)
        return {"red": m - c_black, "black": c_black}

    def transitive_closure(self) -> TransitiveClosure:
        return TransitiveClosure(*warshall(self))


class array(_Avos, ndarray):
    def __new__(cls, *args, **kwargs):
        # unsigned dtypes accept -1 (RED_ONE) by wrapping, as NumPy 1.x did
        if "dtype" in kwargs:
            dt = np.dtype(kwargs["dtype"])
            if dt.kind == "u":
                kw = {k: v for k, v in kwargs.items() if k != "dtype"}
                return asarray(*args, **kw).astype(dt).view(cls)
        return asarray(*args, **kwargs).view(cls)

    def __matmul__(self, other):
        r = super().__matmul__(other)
        return r.view(array) if isinstance(r, ndarray) else r

    def __rmatmul__(self, other):
        r = super().__rmatmul__(other)
        return r.view(array) if isinstance(r, ndarray) else r


def transitive_closure(A: array) -> TransitiveClosure:
    return A.transitive_closure()
