"""Sparse AVOS product on the GPU (redblackgraph/gpu/spgemm.py:32-270): int32 values with the
Cython scalar algebra, optional j >= i mask, sorted output."""
from __future__ import annotations

import time
from typing import Optional

from .. import spgemm as _sp
from .csr_gpu import CSRMatrixGPU


def spgemm(A: CSRMatrixGPU, B: CSRMatrixGPU = None, *, upper_triangular: bool = None) -> CSRMatrixGPU:
    self_multiply = B is None or B is A
    if B is None:
        B = A
    if A.shape[1] != B.shape[0]:
        raise ValueError(f"Incompatible shapes: A is {A.shape}, B is {B.shape}. "
                         f"A.shape[1] must equal B.shape[0].")
    if upper_triangular is None:
        upper_triangular = self_multiply and A.triangular
    C, _, _ = _sp.spgemm(A.device_csr(), B.device_csr(), upper=bool(upper_triangular),
                         sem=_sp.SEM_CY32)
    return CSRMatrixGPU.from_device_csr(C, triangular=bool(upper_triangular))


def spgemm_upper_triangular(A: CSRMatrixGPU, *, validate: bool = True) -> CSRMatrixGPU:
    if A.shape[0] != A.shape[1]:
        raise ValueError(f"Matrix must be square, got {A.shape}")
    if validate and not A.triangular:
        raise ValueError("Matrix must be upper triangular")
    return spgemm(A, upper_triangular=True)


def matmul_gpu(A: CSRMatrixGPU, B: Optional[CSRMatrixGPU] = None) -> CSRMatrixGPU:
    return spgemm(A, B)


class SpGEMMStats:
    """Timing and size statistics of one product (redblackgraph/gpu/spgemm.py:172-230)."""

    def __init__(self, total_time: float, nnz_a: int, nnz_b: int, nnz_c: int, shape):
        self.total_time = total_time
        self.nnz_a, self.nnz_b, self.nnz_c = nnz_a, nnz_b, nnz_c
        self.shape = shape

    def __repr__(self):
        return (f"SpGEMMStats(time={self.total_time * 1e3:.3f} ms, nnz A={self.nnz_a}, "
                f"B={self.nnz_b}, C={self.nnz_c})")


def spgemm_with_stats(A: CSRMatrixGPU, B: CSRMatrixGPU = None, *, upper_triangular: bool = None):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    C = spgemm(A, B, upper_triangular=upper_triangular)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    Bm = A if B is None else B
    return C, SpGEMMStats(t, A.nnz, Bm.nnz, C.nnz, C.shape)
