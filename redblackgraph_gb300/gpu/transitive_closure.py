"""Closures of ``CSRMatrixGPU`` (redblackgraph/gpu/transitive_closure.py:26-652)."""
from __future__ import annotations

from typing import Tuple

import numpy as np
import torch

from .. import _lib
from .. import spgemm as _sp
from .csr_gpu import CSRMatrixGPU


def _max_non_identity(R: CSRMatrixGPU) -> int:
    if R.nnz == 0:
        return 0
    a = R.data.to(torch.int64).abs()
    a = a[a > 1]
    return int(a.max().item()) if a.numel() else 0


def transitive_closure_gpu(A: CSRMatrixGPU, max_iterations: int = 64) -> Tuple[CSRMatrixGPU, int]:
    """R <- R (+) R^2 (the Cython algebra, j >= i when R is triangular, magnitude merge) until
    stable; diameter = max(changing iterations, floor(log2(max |value| > 1)))."""
    if A.nnz == 0:
        return A.copy(), 0
    # the squaring loop in its semi-naive form (same R after every step); the GPU module's
    # products wrap silently, so no step status is raised
    Rd, diameter = _sp.squaring_closure(A.device_csr(), max_iterations, _sp.SEM_CY32, upper=A.triangular,
                                        on_step=lambda rc, flags: None)
    R = CSRMatrixGPU.from_device_csr(Rd, triangular=A.triangular)
    mv = _max_non_identity(R)
    if mv > 1:
        diameter = max(diameter, int(np.floor(np.log2(mv))))
    return R, diameter


def sparse_avos_sum_gpu(A: CSRMatrixGPU, B: CSRMatrixGPU) -> CSRMatrixGPU:
    """Per-cell merge of two matrices: the smaller |value| (A's on a tie), zeros dropped
    (redblackgraph/gpu/transitive_closure.py:77-156), by the GPU row-merge kernel."""
    if A.shape != B.shape:
        raise ValueError(f"Shape mismatch: {A.shape} vs {B.shape}")
    Z = _sp.merge_minabs(A.device_csr(), B.device_csr())
    return CSRMatrixGPU.from_device_csr(Z, triangular=A.triangular and B.triangular)


def sparse_equal_gpu(A: CSRMatrixGPU, B: CSRMatrixGPU) -> bool:
    if A.shape != B.shape or A.nnz != B.nnz:
        return False
    return A.device_csr().equal(B.device_csr())


def transitive_closure_dag_gpu(A: CSRMatrixGPU) -> Tuple[CSRMatrixGPU, int]:
    """Closure of a DAG by topological levels (redblackgraph/gpu/transitive_closure.py:474-652),
    with the level kernels of rbg_dag_closure; diameter = floor(log2(max |value| > 1)) of the
    closure.  Rows too wide for the level kernels take the squaring closure instead."""
    from ..dag import RowTooWide, dag_closure_device
    n = A.shape[0]
    if n == 0 or A.nnz == 0:
        return A.copy(), 0
    try:
        C, _, _ = dag_closure_device(A.device_csr())
        R = CSRMatrixGPU.from_device_csr(C, triangular=A.triangular)
    except RowTooWide:
        R, _ = transitive_closure_gpu(A)
    mv = _max_non_identity(R)
    return R, (int(np.floor(np.log2(mv))) if mv > 1 else 0)
