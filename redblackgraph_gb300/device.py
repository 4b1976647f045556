"""Device plumbing: the CUDA device, the caller's stream, workspaces and host transfers.

PyTorch provides device memory (its caching allocator), streams and pinned host buffers;
all arithmetic happens in ``librbg_gb300.so``.
"""
from __future__ import annotations

import threading

import numpy as np
import torch

_NP_TO_TORCH = {
    np.dtype(np.int8): torch.int8, np.dtype(np.uint8): torch.uint8,
    np.dtype(np.int16): torch.int16, np.dtype(np.uint16): torch.uint16,
    np.dtype(np.int32): torch.int32, np.dtype(np.uint32): torch.uint32,
    np.dtype(np.int64): torch.int64, np.dtype(np.uint64): torch.uint64,
}
_TORCH_TO_NP = {v: k for k, v in _NP_TO_TORCH.items()}


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("redblackgraph_gb300 computes on a CUDA GPU; none is available")
    return torch.device("cuda", torch.cuda.current_device())


def torch_dtype(dtype) -> torch.dtype:
    return _NP_TO_TORCH[np.dtype(dtype)]


def numpy_dtype(dtype: torch.dtype) -> np.dtype:
    return _TORCH_TO_NP[dtype]


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


class Workspace:
    """Grow-only device scratch buffer, one per (device, stream) user."""

    def __init__(self):
        self._buf = None
        self._lock = threading.Lock()

    def get(self, nbytes: int, device: torch.device) -> torch.Tensor:
        with self._lock:
            nbytes = max(int(nbytes), 256)
            if self._buf is None or self._buf.numel() < nbytes or self._buf.device != device:
                self._buf = None
                self._buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
            return self._buf


_default_ws = threading.local()


def default_workspace() -> Workspace:
    """The calling thread's workspace.  Every closure call synchronises its stream before it
    returns, so one thread's calls never overlap on the GPU; calls from different threads (each
    on its own stream) get different buffers and can run at the same time."""
    ws = getattr(_default_ws, "ws", None)
    if ws is None:
        ws = _default_ws.ws = Workspace()
    return ws


def to_device(a: np.ndarray, device: torch.device | None = None,
              stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """Copy a host array to the device as raw bytes (through pinned memory when large) and
    view it with the array's integer dtype; works for every width torch can view."""
    device = device or require_cuda()
    a = np.ascontiguousarray(a)
    raw = torch.from_numpy(a.reshape(-1).view(np.uint8))
    if a.nbytes >= (1 << 20) and not raw.is_pinned():
        raw = raw.pin_memory()
    with torch.cuda.stream(stream) if stream is not None else _nullctx():
        d = raw.to(device, non_blocking=True)
    return d.view(torch_dtype(a.dtype)).reshape(a.shape)


def to_host_pinned(t: torch.Tensor) -> np.ndarray:
    """Copy a device tensor into page-locked host memory (a fast device-to-host copy); the
    returned array keeps that memory alive."""
    npdt = numpy_dtype(t.dtype)
    src = t.contiguous().reshape(-1).view(torch.uint8)
    dst = torch.empty(src.numel(), dtype=torch.uint8, pin_memory=True)
    dst.copy_(src)
    return dst.numpy().view(npdt).reshape(tuple(t.shape))


def csr_from_parts(data: np.ndarray, indices: np.ndarray, indptr: np.ndarray, shape, canonical: bool = True,
                   cls=None):
    """A scipy CSR matrix over these host arrays as they are: the library's outputs are already
    valid CSR (sorted rows, no duplicates), so the constructor's checks and copies are skipped.
    The index arrays share one dtype (int32 when the entries fit, else int64).  ``cls`` is a
    csr_matrix subclass to build (default csr_matrix)."""
    import scipy.sparse as sp
    idx = np.int32 if indptr.size == 0 or int(indptr[-1]) < 2**31 - 1 else np.int64
    m = (cls or sp.csr_matrix)(tuple(shape), dtype=data.dtype)
    m.data = data
    m.indices = indices if indices.dtype == idx else indices.astype(idx)
    m.indptr = indptr if indptr.dtype == idx else indptr.astype(idx)
    if canonical:
        m.has_sorted_indices = True
        m.has_canonical_format = True
    return m


def to_host(t: torch.Tensor) -> np.ndarray:
    npdt = numpy_dtype(t.dtype)
    raw = t.contiguous().reshape(-1).view(torch.uint8).cpu().numpy()
    return raw.view(npdt).reshape(tuple(t.shape))


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
