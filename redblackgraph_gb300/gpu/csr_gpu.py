"""``CSRMatrixGPU``: a CSR matrix resident on the GPU (redblackgraph/gpu/csr_gpu.py:32-334).

Data are int32 (as the reference forces), indices int32, row pointers int64 on the device.
Arrays are torch tensors; every product and closure runs in librbg_gb300.so.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import torch

from ..spgemm import DeviceCSR
from ..device import require_cuda, to_device, to_host


class CSRMatrixGPU:
    def __init__(self, data, indices, indptr, shape: Tuple[int, int], *, triangular: bool = False,
                 validate: bool = True):
        dev = require_cuda()
        self.data = _as_tensor(data, torch.int32, dev)
        self.indices = _as_tensor(indices, torch.int32, dev)
        self.indptr = _as_tensor(indptr, torch.int64, dev)
        self.shape = tuple(shape)
        self.triangular = triangular
        if validate:
            self._validate_csr()
            if triangular:
                self._validate_triangular()

    # ------------------------------------------------------------------ validation
    def _validate_csr(self):
        rows, cols = self.shape
        nnz = self.data.numel()
        if self.indices.numel() != nnz:
            raise ValueError(f"indices length {self.indices.numel()} != data length {nnz}")
        if self.indptr.numel() != rows + 1:
            raise ValueError(f"indptr length {self.indptr.numel()} != rows + 1 ({rows + 1})")
        if rows > 0 and bool((self.indptr[1:] < self.indptr[:-1]).any()):
            raise ValueError("indptr is not monotonically non-decreasing")
        if int(self.indptr[0]) != 0:
            raise ValueError(f"indptr[0] should be 0, got {int(self.indptr[0])}")
        if int(self.indptr[-1]) != nnz:
            raise ValueError(f"indptr[-1] should be {nnz}, got {int(self.indptr[-1])}")
        if nnz and (bool((self.indices < 0).any()) or bool((self.indices >= cols).any())):
            raise ValueError(f"Column indices out of bounds [0, {cols})")

    def _rows(self):
        return torch.repeat_interleave(torch.arange(self.shape[0], device=self.indptr.device),
                                       self.indptr[1:] - self.indptr[:-1])

    def _validate_triangular(self):
        if self.nnz and bool((self.indices.to(torch.int64) < self._rows()).any()):
            raise ValueError("Not upper triangular")

    # ------------------------------------------------------------------ conversion
    @classmethod
    def from_cpu(cls, cpu_matrix, *, triangular: Optional[bool] = None, validate: bool = True):
        import scipy.sparse as sp
        m = cpu_matrix.tocsr() if not sp.isspmatrix_csr(cpu_matrix) else cpu_matrix
        if triangular is None:
            rows = np.repeat(np.arange(m.shape[0]), np.diff(m.indptr))
            triangular = bool(np.all(m.indices >= rows))
        return cls(np.asarray(m.data).astype(np.int32), np.asarray(m.indices).astype(np.int32),
                   np.asarray(m.indptr).astype(np.int64), m.shape, triangular=triangular,
                   validate=validate)

    def to_cpu(self):
        return self.device_csr().to_scipy()

    def device_csr(self) -> DeviceCSR:
        return DeviceCSR(self.indptr, self.indices, self.data, self.shape)

    @classmethod
    def from_device_csr(cls, c: DeviceCSR, triangular: bool = False):
        return cls(c.data.to(torch.int32), c.indices, c.indptr, c.shape, triangular=triangular,
                   validate=False)

    # ------------------------------------------------------------------ properties / ops
    @property
    def nnz(self) -> int:
        return int(self.data.numel())

    @property
    def dtype(self):
        return np.dtype(np.int32)

    def __matmul__(self, other):
        from .spgemm import spgemm
        if not isinstance(other, CSRMatrixGPU):
            return NotImplemented
        return spgemm(self, other)

    def copy(self):
        return CSRMatrixGPU(self.data.clone(), self.indices.clone(), self.indptr.clone(), self.shape,
                            triangular=self.triangular, validate=False)

    def eliminate_zeros(self):
        keep = self.data != 0
        if bool(keep.all()):
            return
        counts = torch.zeros(self.shape[0] + 1, dtype=torch.int64, device=self.data.device)
        counts[1:] = torch.segment_reduce(keep.to(torch.int64), "sum",
                                          lengths=self.indptr[1:] - self.indptr[:-1])
        self.data = self.data[keep]
        self.indices = self.indices[keep]
        self.indptr = torch.cumsum(counts, 0)

    def transitive_closure(self, max_iterations=64):
        from .transitive_closure import transitive_closure_gpu
        return transitive_closure_gpu(self, max_iterations=max_iterations)

    def prefetch(self, device=None):
        """The arrays are device-resident already (no managed memory is used)."""
        return None

    def __repr__(self) -> str:
        tri = " (upper triangular)" if self.triangular else ""
        return f"CSRMatrixGPU({self.shape[0]}x{self.shape[1]}, nnz={self.nnz}{tri})"

    def memory_usage(self) -> dict:
        d = self.data.numel() * 4
        i = self.indices.numel() * 4
        p = self.indptr.numel() * 8
        t = d + i + p
        return {"data": d, "indices": i, "indptr": p, "total": t,
                "total_mb": t / 1024 ** 2, "total_gb": t / 1024 ** 3}


def _as_tensor(x, dtype, dev):
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=dtype) if (x.dtype != dtype or x.device != dev) else x
    return to_device(np.ascontiguousarray(np.asarray(x), dtype=np.dtype(str(dtype).split(".")[-1])), dev)


def validate_triangular_mask(i: int, j: int) -> bool:
    return j >= i
