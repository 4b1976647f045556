"""``rb_matrix``: scipy CSR with the AVOS product (redblackgraph/sparse/rbm.py:10-122).

``@`` / ``*`` (matrix operands) run the sparse AVOS product on the GPU with the reference's
semantics: inputs canonicalised (sorted, duplicates summed), values widened to 64 bits for the
product (unsigned RED_ONE widened to all ones), zero sums dropped, result cast back to the
operands' common dtype.  Column indices come out sorted within each row; the reference's own
pass 2 emits them in its accumulator's order, so results compare equal as matrices.
"""
from __future__ import annotations

import numpy as np
from scipy.sparse import csr_matrix

from .. import _lib


class rb_matrix(csr_matrix):

    def __matmul__(self, other):
        return self._mul_sparse_matrix(other)

    def __rmatmul__(self, other):
        return self.__class__(other)._mul_sparse_matrix(self)

    def __mul__(self, other):
        if np.isscalar(other):
            return super().__mul__(other)
        return self._mul_sparse_matrix(other)

    def __rmul__(self, other):
        if np.isscalar(other):
            return super().__rmul__(other)
        return self.__class__(other)._mul_sparse_matrix(self)

    def transitive_closure(self, method="D"):
        from .csgraph import transitive_closure
        return transitive_closure(self, method)

    def _mul_sparse_matrix(self, other):
        from ..spgemm import DeviceCSR, spgemm, SEM_C64
        other = self.__class__(other)
        M, K1 = self.shape
        K2, N = other.shape
        if K1 != K2:
            raise ValueError("dimension mismatch")
        a = csr_matrix(self, copy=True)
        b = csr_matrix(other, copy=True)
        for m in (a, b):
            m.sort_indices()
            m.sum_duplicates()
        out_dtype = np.promote_types(a.dtype, b.dtype)
        if out_dtype.kind not in "iu":
            raise TypeError(f"AVOS product needs integer matrices, got {out_dtype}")
        if out_dtype.itemsize < 4:
            work = np.dtype(np.uint32) if out_dtype.kind == "u" else np.dtype(np.int32)
        else:
            work = out_dtype

        def widen(m):
            d = np.asarray(m.data)
            w = d.astype(work)
            if out_dtype.kind == "u" and d.dtype.itemsize < work.itemsize:
                w[d == np.iinfo(d.dtype).max] = np.iinfo(work).max   # RED_ONE stays all ones
            return w

        A = DeviceCSR.from_scipy(csr_matrix((widen(a), a.indices, a.indptr), shape=a.shape))
        B = DeviceCSR.from_scipy(csr_matrix((widen(b), b.indices, b.indptr), shape=b.shape))
        C, rc, flags = spgemm(A, B, sem=SEM_C64, out_dtype=work)
        if rc == _lib.RBG_ERR_OVERFLOW:
            raise OverflowError("Avos product results in an overflow.")
        res = C.to_scipy()
        data = res.data.astype(out_dtype) if res.data.dtype != out_dtype else res.data
        return rb_matrix((data, res.indices, res.indptr), shape=(M, N))
