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

__all__ = ["array", "transitive_closure", "warshall", "vertex_relational_composition",
           "edge_relational_composition"]


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

    def vertex_relational_composition(self, u, v, c, compute_closure=False):
        """The closure with a new vertex lambda (row u, column v, colour c) added to this closure
        (redblack.py:52-75): one rbg_vertex_compose on the GPU.  ValueError when lambda closes
        a cycle, OverflowError when a product overflows, as the C core raises."""
        from ..composition import vertex_compose_host
        R_star = warshall(self)[0] if compute_closure else self
        u, v = np.asarray(u), np.asarray(v)
        if len(u.shape) > 1:
            u = u.reshape((1, R_star.shape[0]))[0]
        if len(v.shape) > 1:
            v = v.reshape((1, R_star.shape[1]))[0]
        loop = _loop_dtype(u, R_star, v)
        out = vertex_compose_host(u.astype(loop), np.asarray(R_star).astype(loop), v.astype(loop), c)
        return out.astype(np.asarray(R_star).dtype, copy=False).view(type(self))

    def edge_relational_composition(self, alpha, beta, relationship, compute_closure=False):
        """The closure with the edge alpha -> beta of value ``relationship`` added
        (redblack.py:77-97): one rbg_edge_compose on the GPU."""
        from ..composition import edge_compose_host
        R_star = warshall(self)[0] if compute_closure else self
        if R_star[beta][alpha] != 0:
            raise ValueError("Relational composition would result in a cycle.")
        return edge_compose_host(np.asarray(R_star), alpha, beta, relationship).view(type(self))


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


def _loop_dtype(*arrays) -> np.dtype:
    """The integer storage type the gufunc's loop runs in: the common type of the operands
    (no integer loop takes int64 and uint64 together)."""
    dt = np.result_type(*[np.asarray(a).dtype for a in arrays])
    if dt.kind not in "iu":
        raise TypeError(f"no relational composition loop for {[np.asarray(a).dtype.name for a in arrays]}")
    return dt


def vertex_relational_composition(u, A: array, v, c, compute_closure=False):
    return A.vertex_relational_composition(u, v, c, compute_closure=compute_closure)


def edge_relational_composition(A: array, alpha, beta, relationship, compute_closure=False):
    return A.edge_relational_composition(alpha, beta, relationship, compute_closure=compute_closure)
