"""Sparse AVOS product and squaring closure on the GPU, at the device-tensor level.

``DeviceCSR`` holds a CSR matrix in device memory (int64 row pointers, int32 column indices,
integer values); ``spgemm`` runs the three-step C ABI (rbg_spgemm_count / _numeric / _gather,
include/rbg_gb300.h); ``squaring_closure`` iterates R <- R (+) R^2 until R stops changing.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import numpy_dtype, require_cuda, stream_handle, to_device, to_host, torch_dtype

SEM_C64 = 0     # rb_matrix @ : C core algebra on 64-bit values, cast back to the storage type
SEM_CY32 = 1    # redblackgraph.gpu : int32 values with the Cython algebra


RbgCsr = _lib.RbgCsr


@dataclass
class DeviceCSR:
    indptr: torch.Tensor    # int64, n_rows + 1
    indices: torch.Tensor   # int32, nnz
    data: torch.Tensor      # integer values, nnz
    shape: tuple

    @property
    def nnz(self) -> int:
        return int(self.indices.numel())

    def cstruct(self) -> RbgCsr:
        return RbgCsr(self.shape[0], self.shape[1], self.indptr.data_ptr(),
                      self.indices.data_ptr() if self.nnz else self.indptr.data_ptr(),
                      self.data.data_ptr() if self.nnz else self.indptr.data_ptr())

    @classmethod
    def from_scipy(cls, m, dtype=None, device=None) -> "DeviceCSR":
        import scipy.sparse as sp
        m = sp.csr_matrix(m)
        if not m.has_sorted_indices:
            m = m.copy()
            m.sort_indices()
        dev = device or require_cuda()
        data = np.ascontiguousarray(m.data, dtype=dtype or m.data.dtype)
        return cls(to_device(np.ascontiguousarray(m.indptr, dtype=np.int64), dev),
                   to_device(np.ascontiguousarray(m.indices, dtype=np.int32), dev),
                   to_device(data, dev), tuple(m.shape))

    def to_scipy(self, cls=None):
        """The matrix on the host (rows as stored; no constructor copies)."""
        from .device import csr_from_parts
        return csr_from_parts(to_host(self.data), to_host(self.indices), to_host(self.indptr), self.shape,
                              canonical=False, cls=cls)

    def equal(self, other: "DeviceCSR") -> bool:
        """Same pattern and values (compared as values, whatever the two dtypes)."""
        if self.shape != other.shape or self.nnz != other.nnz:
            return False
        if not (torch.equal(self.indptr, other.indptr) and torch.equal(self.indices, other.indices)):
            return False
        if self.data.dtype == other.data.dtype:
            return torch.equal(self.data, other.data)
        return torch.equal(self.data.to(torch.int64), other.data.to(torch.int64))


def spgemm(A: DeviceCSR, B: DeviceCSR, R: DeviceCSR | None = None, upper: bool = False,
           sem: int = SEM_C64, out_dtype=None, stream=None, stats: dict | None = None
           ) -> tuple[DeviceCSR, int, int]:
    """C = A (x) B (or the squaring step R (+) R^2 when R is given).

    Returns ``(C, status, flags)``; status is RBG_OK or RBG_ERR_OVERFLOW (C core semantics).
    ``stats``, when given, receives the number of products (A entry x B row entry) and of rows
    taking the dense accumulator.
    """
    if A.shape[1] != B.shape[0]:
        raise ValueError(f"Incompatible shapes: A is {A.shape}, B is {B.shape}.")
    dev = A.indptr.device
    L = _lib.load()
    dt = numpy_dtype(A.data.dtype)
    code = _lib.dtype_code(dt)
    n, nc = A.shape[0], B.shape[1]
    ca, cb = A.cstruct(), B.cstruct()
    cr = R.cstruct() if R is not None else None
    hb = ctypes.c_int64(0)
    _lib.check(L.rbg_spgemm_head_bytes(n, ctypes.byref(hb)), "spgemm")
    head = torch.empty(max(hb.value, 256), dtype=torch.uint8, device=dev)
    tot, dense = ctypes.c_int64(0), ctypes.c_int64(0)
    sh = stream_handle(stream)
    _lib.check(L.rbg_spgemm_count(ctypes.byref(ca), ctypes.byref(cb),
                                  ctypes.byref(cr) if cr is not None else None, int(upper),
                                  head.data_ptr(), head.numel(), ctypes.byref(tot),
                                  ctypes.byref(dense), sh), "spgemm_count")
    if stats is not None:
        stats["products"] = tot.value - (R.nnz if R is not None else 0)
        stats["dense_rows"] = dense.value
    tb = ctypes.c_int64(0)
    _lib.check(L.rbg_spgemm_tail_bytes(n, nc, tot.value, dense.value, ctypes.byref(tb)), "spgemm")
    tail = torch.empty(max(tb.value, 256), dtype=torch.uint8, device=dev)
    nnz, flags = ctypes.c_int64(0), ctypes.c_uint32(0)
    rc = L.rbg_spgemm_numeric(sem, code, ctypes.byref(ca), ctypes.byref(cb),
                              ctypes.byref(cr) if cr is not None else None, int(upper),
                              head.data_ptr(), tail.data_ptr(), tail.numel(), tot.value, dense.value,
                              ctypes.byref(nnz), ctypes.byref(flags), sh)
    if rc not in (_lib.RBG_OK, _lib.RBG_ERR_OVERFLOW):
        _lib.check(rc, "spgemm_numeric")
    odt = np.dtype(np.int32) if R is not None else np.dtype(out_dtype or dt)
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
    data = torch.empty(max(nnz.value, 1), dtype=torch_dtype(odt), device=dev)[:nnz.value]
    _lib.check(L.rbg_spgemm_gather(_lib.dtype_code(odt), n, nc, head.data_ptr(), tail.data_ptr(),
                                   tot.value, dense.value, indptr.data_ptr(),
                                   indices.data_ptr() if nnz.value else indptr.data_ptr(),
                                   data.data_ptr() if nnz.value else indptr.data_ptr(), sh),
               "spgemm_gather")
    return DeviceCSR(indptr, indices, data, (n, nc)), rc, flags.value


def csr_diff(X: DeviceCSR, Y: DeviceCSR, stream=None) -> DeviceCSR:
    """The entries of X that Y does not hold with the same value (rbg_csr_diff_count / _fill),
    in X's storage type."""
    if X.shape != Y.shape:
        raise ValueError(f"Shape mismatch: {X.shape} vs {Y.shape}")
    dev = X.indptr.device
    L = _lib.load()
    cx, cy = X.cstruct(), Y.cstruct()
    xd = _lib.dtype_code(numpy_dtype(X.data.dtype))
    yd = _lib.dtype_code(numpy_dtype(Y.data.dtype))
    hb = ctypes.c_int64(0)
    _lib.check(L.rbg_spgemm_head_bytes(X.shape[0], ctypes.byref(hb)), "diff")
    head = torch.empty(max(hb.value, 256), dtype=torch.uint8, device=dev)
    nnz = ctypes.c_int64(0)
    sh = stream_handle(stream)
    _lib.check(L.rbg_csr_diff_count(xd, ctypes.byref(cx), yd, ctypes.byref(cy), head.data_ptr(), head.numel(),
                                    ctypes.byref(nnz), sh), "diff_count")
    n = X.shape[0]
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
    data = torch.empty(max(nnz.value, 1), dtype=X.data.dtype, device=dev)[:nnz.value]
    _lib.check(L.rbg_csr_diff_fill(xd, ctypes.byref(cx), yd, ctypes.byref(cy), head.data_ptr(), indptr.data_ptr(),
                                   indices.data_ptr() if nnz.value else indptr.data_ptr(),
                                   data.data_ptr() if nnz.value else indptr.data_ptr(), sh), "diff_fill")
    return DeviceCSR(indptr, indices, data, X.shape)


def seminaive_operands(D: DeviceCSR, R: DeviceCSR, stream=None) -> tuple[DeviceCSR, DeviceCSR]:
    """A' = [D R] and B' = [R ; D] (rbg_spgemm_seminaive_operands): A' B' = D R (+) R D."""
    if D.shape != R.shape or R.shape[0] != R.shape[1]:
        raise ValueError("D and R must be square and of one shape")
    if D.data.dtype != R.data.dtype:
        raise ValueError("D and R must hold one value type")
    n = R.shape[0]
    dev = R.indptr.device
    m = D.nnz + R.nnz
    a_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    b_indptr = torch.empty(2 * n + 1, dtype=torch.int64, device=dev)
    a_ind = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    b_ind = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    a_dat = torch.empty(max(m, 1), dtype=R.data.dtype, device=dev)
    b_dat = torch.empty(max(m, 1), dtype=R.data.dtype, device=dev)
    cd, cr = D.cstruct(), R.cstruct()
    _lib.check(_lib.load().rbg_spgemm_seminaive_operands(
        _lib.dtype_code(numpy_dtype(R.data.dtype)), ctypes.byref(cd), ctypes.byref(cr), a_indptr.data_ptr(),
        a_ind.data_ptr(), a_dat.data_ptr(), b_indptr.data_ptr(), b_ind.data_ptr(), b_dat.data_ptr(),
        stream_handle(stream)), "seminaive_operands")
    return (DeviceCSR(a_indptr, a_ind[:m], a_dat[:m], (n, 2 * n)),
            DeviceCSR(b_indptr, b_ind[:m], b_dat[:m], (2 * n, n)))


def squaring_closure(A: DeviceCSR, max_iterations: int = 64, sem: int = SEM_C64, upper: bool = False,
                     on_step=None, stream=None, steps: list | None = None,
                     seminaive: bool = False) -> tuple[DeviceCSR, int]:
    """R <- R (+) R^2 until R stops changing (at most ``max_iterations`` steps).

    ``seminaive`` selects the semi-naive form of a step, which gives the same R: with D the
    entries the previous step changed, a product of two entries outside D was already formed by
    that step and folded into R, so R (+) R^2 = R (+) D R (+) R D (the (+) is a minimum and (x) is
    monotone in each operand, hence distributes over it).  A step takes that form when D holds at
    most half of R's entries, as the one product [D R] [R ; D] merged with R, and D comes from
    rbg_csr_diff (which also tests convergence).  It forms fewer products, but each step still
    merges and rewrites all of R and computes D, which on pedigree forests costs more than the
    products it saves, so the plain loop (convergence by comparing R) is the default.
    ``on_step(status, flags)`` sees each step's product status and event flags (it may raise);
    ``steps``, when given, receives per step (form, products, nnz in, nnz out).

    Returns ``(R, steps that changed R)``; R is the last step's output (int32 values).
    """
    R, D = A, None
    changed = 0
    for _ in range(max_iterations):
        st = {}
        if not seminaive or D is None or 2 * D.nnz > R.nnz:
            Rn, rc, fl = spgemm(R, R, R=R, upper=upper, sem=sem, stream=stream, stats=st)
            prods, form = st["products"], "square"
        else:
            A2, B2 = seminaive_operands(D, R, stream=stream)
            Rn, rc, fl = spgemm(A2, B2, R=R, upper=upper, sem=sem, stream=stream, stats=st)
            prods, form = st["products"], "semi-naive"
        if on_step is not None:
            on_step(rc, fl)
        elif rc == _lib.RBG_ERR_OVERFLOW:
            raise OverflowError("Avos product results in an overflow.")
        if steps is not None:
            steps.append((form, prods, R.nnz, Rn.nnz))
        if seminaive:
            D = csr_diff(Rn, R, stream=stream)
            stable = D.nnz == 0
        else:
            stable = Rn.equal(R)
        R = Rn
        if stable:
            break
        changed += 1
    return R, changed


def merge_minabs(X: DeviceCSR, Y: DeviceCSR, stream=None) -> DeviceCSR:
    """Z = X (+) Y with the magnitude rule (int32 values), on the GPU."""
    if X.shape != Y.shape:
        raise ValueError(f"Shape mismatch: {X.shape} vs {Y.shape}")
    dev = X.indptr.device
    L = _lib.load()
    cx, cy = X.cstruct(), Y.cstruct()
    hb = ctypes.c_int64(0)
    _lib.check(L.rbg_spgemm_head_bytes(X.shape[0], ctypes.byref(hb)), "merge")
    head = torch.empty(max(hb.value, 256), dtype=torch.uint8, device=dev)
    nnz = ctypes.c_int64(0)
    sh = stream_handle(stream)
    _lib.check(L.rbg_csr_merge_count(ctypes.byref(cx), ctypes.byref(cy), head.data_ptr(), head.numel(),
                                     ctypes.byref(nnz), sh), "merge_count")
    n = X.shape[0]
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
    data = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
    _lib.check(L.rbg_csr_merge_fill(ctypes.byref(cx), ctypes.byref(cy), head.data_ptr(), indptr.data_ptr(),
                                    indices.data_ptr() if nnz.value else indptr.data_ptr(),
                                    data.data_ptr() if nnz.value else indptr.data_ptr(), sh), "merge_fill")
    return DeviceCSR(indptr, indices, data, X.shape)
