"""GPU sparse AVOS operations (the ``redblackgraph.gpu`` surface, redblackgraph/gpu/__init__.py).

``CUPY_AVAILABLE`` is kept for callers that test it: here it reports whether a CUDA device and
the native library are usable.
"""
__all__ = ["CSRMatrixGPU", "spgemm", "spgemm_upper_triangular", "matmul_gpu",
           "transitive_closure_gpu", "transitive_closure_dag_gpu", "CUPY_AVAILABLE"]


def _available() -> bool:
    try:
        import torch
        from .. import _lib
        _lib.load()
        return torch.cuda.is_available()
    except Exception:
        return False


CUPY_AVAILABLE = _available()

from .csr_gpu import CSRMatrixGPU  # noqa: E402
from .spgemm import spgemm, spgemm_upper_triangular, matmul_gpu, spgemm_with_stats, SpGEMMStats  # noqa: E402
from .transitive_closure import transitive_closure_gpu, transitive_closure_dag_gpu  # noqa: E402
