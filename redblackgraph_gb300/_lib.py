"""ctypes binding of ``librbg_gb300.so`` -- the only way the Python layer reaches the GPU.

The library is the product: there is no CPU fallback.  Loading fails loudly when the
library has not been built, and every call that needs a device fails loudly without one.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "librbg_gb300.so"

# dtype codes (include/rbg_gb300.h)
DTYPE_CODE = {
    np.dtype(np.int8): 0, np.dtype(np.uint8): 1, np.dtype(np.int16): 2, np.dtype(np.uint16): 3,
    np.dtype(np.int32): 4, np.dtype(np.uint32): 5, np.dtype(np.int64): 6, np.dtype(np.uint64): 7,
}

RBG_OK = 0
RBG_ERR_OVERFLOW = 1
RBG_ERR_CYCLE = 2
RBG_ERR_CAPACITY = 3
RBG_ERR_NOMEM = 4
RBG_ERR_TIMEOUT = 5
RBG_ERR_INVALID = 6
RBG_ERR_CUDA = -1

EV_OVF_SIZE, EV_OVF_ONES, EV_HANG, EV_CYCLE = 1, 2, 4, 8

MODE_CYTHON = 1
MODE_TRIANGULAR = 2
MODE_FORCE_EXACT = 4
MODE_FORCE_WIDE = 8
MODE_GRAPH = 16
MODE_TILE_NARROW = 32
MODE_AUTOTUNE = 64
MODE_NO_DAG = 128

PATH_BLOCKED32, PATH_BLOCKED64, PATH_EXACT, PATH_DAG = 1, 2, 3, 4

NOALLOC_MAX_N = 1024   # include/rbg_gb300.h RBG_NOALLOC_MAX_N


class RbgResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("flags", ctypes.c_uint32),
        ("diameter", ctypes.c_int64),
        ("k", ctypes.c_int64),
        ("i", ctypes.c_int64),
        ("j", ctypes.c_int64),
        ("path", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("executed", ctypes.c_int64),
    ]


# the same record as a numpy structured dtype (results of a batch read without per-item objects)
RESULT_DTYPE = np.dtype([("status", "<i4"), ("flags", "<u4"), ("diameter", "<i8"), ("k", "<i8"),
                         ("i", "<i8"), ("j", "<i8"), ("path", "<i4"), ("reserved", "<i4"),
                         ("executed", "<i8")])


class RbgCsr(ctypes.Structure):
    """rbg_csr_t: a device CSR matrix (int64 row pointers, int32 indices, values)."""
    _fields_ = [("n_rows", ctypes.c_int64), ("n_cols", ctypes.c_int64),
                ("indptr", ctypes.c_void_p), ("indices", ctypes.c_void_p),
                ("data", ctypes.c_void_p)]


class RbgLookup(ctypes.Structure):
    """rbg_lookup_t: one relationship query on a resident closed matrix."""
    _fields_ = [("W", ctypes.c_void_p), ("ld", ctypes.c_int64), ("rows", ctypes.c_int64),
                ("n", ctypes.c_int64), ("u", ctypes.c_int64), ("v", ctypes.c_int64),
                ("dtype", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RbgComposeResult(ctypes.Structure):
    """rbg_compose_result_t: outcome of a relational composition."""
    _fields_ = [("status", ctypes.c_int32), ("flags", ctypes.c_uint32), ("event", ctypes.c_uint32),
                ("reserved", ctypes.c_int32), ("step", ctypes.c_int64), ("i", ctypes.c_int64),
                ("j", ctypes.c_int64), ("lhs", ctypes.c_int64), ("rhs", ctypes.c_int64),
                ("updated", ctypes.c_int64)]


class RbgRowStats(ctypes.Structure):
    """rbg_row_stats_t: where rbg_fw_batch_rows records per-row statistics (device pointers)."""
    _fields_ = [("row_base", ctypes.c_void_p), ("row_id", ctypes.c_void_p), ("row_count", ctypes.c_void_p),
                ("chunk_mask", ctypes.c_void_p), ("comp_max", ctypes.c_void_p)]


# (name, restype, argtypes) of every exported entry point; include/rbg_gb300.h declares them
_P = ctypes.c_void_p
_I32, _U32, _I64 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_int64
SIGNATURES = [
    ("rbg_version", _I32, []),
    ("rbg_launch_count", _I64, []),
    ("rbg_profile_begin", _I32, []),
    ("rbg_profile_end", _I32, [_P, _P]),
    ("rbg_profile_end_slots", _I32, [_P, _P, _I32]),
    ("rbg_fw_dense_workspace_bytes", _I32, [_I32, _I64, _U32, ctypes.POINTER(_I64)]),
    ("rbg_fw_dense", _I32, [_I32, _I64, _P, _I64, _P, _I64, _U32, _P, _I64,
                            ctypes.POINTER(RbgResult), _P]),
    ("rbg_fw_dense_noalloc", _I32, [_I32, _I64, _P, _I64, _P, _I64, _U32,
                                    ctypes.POINTER(RbgResult), _P]),
    ("rbg_fw_batch_workspace_bytes", _I32, [_I32, _I64, _P, _U32, ctypes.POINTER(_I64)]),
    ("rbg_fw_batch", _I32, [_I32, _I64, _P, _P, _P, _P, _U32, _P, _I64, _P, _P]),
    ("rbg_release_scratch", _I32, []),
    ("rbg_fw_batch_rows", _I32, [_I32, _I64, _P, _P, _P, _P, _U32, _P, _I64, ctypes.POINTER(RbgRowStats), _P, _P]),
    ("rbg_spgemm_head_bytes", _I32, [_I64, ctypes.POINTER(_I64)]),
    ("rbg_spgemm_count", _I32, [ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr),
                                _I32, _P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_I64), _P]),
    ("rbg_spgemm_tail_bytes", _I32, [_I64, _I64, _I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_spgemm_numeric", _I32, [_I32, _I32, ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr),
                                  ctypes.POINTER(RbgCsr), _I32, _P, _P, _I64, _I64, _I64,
                                  ctypes.POINTER(_I64), ctypes.POINTER(_U32), _P]),
    ("rbg_spgemm_gather", _I32, [_I32, _I64, _I64, _P, _P, _I64, _I64, _P, _P, _P, _P]),
    ("rbg_csr_merge_count", _I32, [ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr), _P, _I64,
                                   ctypes.POINTER(_I64), _P]),
    ("rbg_csr_merge_fill", _I32, [ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr), _P, _P, _P, _P, _P]),
    ("rbg_csr_diff_count", _I32, [_I32, ctypes.POINTER(RbgCsr), _I32, ctypes.POINTER(RbgCsr), _P, _I64,
                                  ctypes.POINTER(_I64), _P]),
    ("rbg_csr_diff_fill", _I32, [_I32, ctypes.POINTER(RbgCsr), _I32, ctypes.POINTER(RbgCsr), _P, _P, _P, _P,
                                 _P]),
    ("rbg_spgemm_seminaive_operands", _I32, [_I32, ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr), _P, _P, _P,
                                             _P, _P, _P, _P]),
    ("rbg_avos_matmul_workspace_bytes", _I32, [_I32, _I64, _I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_avos_matmul", _I32, [_I32, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _P, _I64,
                               ctypes.POINTER(_U32), _P]),
    ("rbg_avos_elementwise", _I32, [_I32, _I32, _I64, _P, _P, _P, _P, _I64, ctypes.POINTER(_U32), _P]),
    ("rbg_cc_workspace_bytes", _I32, [_I64, ctypes.POINTER(_I64)]),
    ("rbg_cc_label", _I32, [_I64, _P, _P, _P, _I64, _P, _P, _P, _P, ctypes.POINTER(_I64), _P]),
    ("rbg_cc_densify", _I32, [_I32, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _I64, _P]),
    ("rbg_cc_chunk_mask_words", _I32, [_I64, _I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_cc_compact_count", _I32, [_I64, _I64, _P, _P, _P, _P, _P, _P, _I64, ctypes.POINTER(_I64), _P, _P, _P]),
    ("rbg_cc_compact_scan", _I32, [_I64, _P, _P, _I64, ctypes.POINTER(_I64), _P]),
    ("rbg_cc_dag_classify", _I32, [_I64, _P, _P, _P, _P, _P, _I64, _P, _I64, _P, _P, _P, ctypes.POINTER(_I64), _P]),
    ("rbg_cc_dag_edges", _I32, [_I64, _P, _P, _P, _P, _P, _P, _P]),
    ("rbg_cc_dag_stats", _I32, [_I64, _I64, _P, _P, _P, _P, _P, ctypes.POINTER(RbgCsr), _P, _P, _P, _P, _P,
                                _P, _P, _P, _P]),
    ("rbg_cc_dag_merge_count", _I32, [_I64, _P, _P, _P, _I64, _P, ctypes.POINTER(_I64), _P]),
    ("rbg_cc_dag_merge_fill", _I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("rbg_cc_compact_fill", _I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("rbg_relationship_lookup", _I32, [_I64, _P, _P, _P]),
    ("rbg_dag_workspace_bytes", _I32, [_I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_dag_closure", _I32, [ctypes.POINTER(RbgCsr), _P, _I64, _P, _P, _I64, _P, _P, ctypes.POINTER(_I64),
                               ctypes.POINTER(_I64), ctypes.POINTER(_I64), _P]),
    ("rbg_dag_gather_workspace_bytes", _I32, [_I64, ctypes.POINTER(_I64)]),
    ("rbg_dag_gather", _I32, [_I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    ("rbg_dag_candidate_max", _I32, [ctypes.POINTER(RbgCsr), ctypes.POINTER(RbgCsr), _P, _I64,
                                     ctypes.POINTER(_I64), _P]),
    ("rbg_compose_workspace_bytes", _I32, [_I32, _I64, ctypes.POINTER(_I64)]),
    ("rbg_vertex_compose", _I32, [_I32, _I64, _P, _I64, _P, _P, _I64, _P, _I64, _U32, _P, _I64,
                                  ctypes.POINTER(RbgComposeResult), _P]),
    ("rbg_edge_compose", _I32, [_I32, _I64, _P, _I64, _I64, _I64, _I64, _P, _I64, _U32, _P, _I64,
                                ctypes.POINTER(RbgComposeResult), _P]),
    ("rbg_ordering_metrics_csr", _I32, [_I64, _P, _P, _P, _P, _P, _P, _P]),
    ("rbg_ordering_metrics_dense", _I32, [_I64, _P, _I64, _P, _P, _P, _P]),
    ("rbg_canonical_permutation_workspace_bytes", _I32, [_I64, ctypes.POINTER(_I64)]),
    ("rbg_canonical_permutation", _I32, [_I64, _P, _P, _P, _P, _P, _P, _P, _I64, _P]),
    ("rbg_permute_dense", _I32, [_I32, _I64, _P, _I64, _P, _P, _I64, _I32, _P]),
    ("rbg_permute_csr_workspace_bytes", _I32, [_I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_permute_csr_count", _I32, [ctypes.POINTER(RbgCsr), _P, _I32, _P, _P, _I64, ctypes.POINTER(_I64), _P]),
    ("rbg_permute_csr_fill", _I32, [ctypes.POINTER(RbgCsr), _P, _I32, _P, _P, _P, _P, _I64, _P]),
    ("rbg_topological_workspace_bytes", _I32, [_I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_topological_order", _I32, [ctypes.POINTER(RbgCsr), _P, _I64, _P, ctypes.POINTER(_I64),
                                     ctypes.POINTER(_I64), _P]),
    ("rbg_is_upper_triangular_csr", _I32, [ctypes.POINTER(RbgCsr), _I32, ctypes.POINTER(_I32), _P, _I64, _P]),
    ("rbg_csr_remap_workspace_bytes", _I32, [_I64, _I64, ctypes.POINTER(_I64)]),
    ("rbg_csr_remap", _I32, [ctypes.POINTER(RbgCsr), _P, _P, _I64, _P, _P, _P, _I64, _P, _I64,
                             ctypes.POINTER(_I64), _P]),
]

_lib = None


def load(path: Path | None = None) -> ctypes.CDLL:
    """Load (once) and declare the native library; raises when it is missing."""
    global _lib
    if _lib is None:
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"native library {p} is missing: build it with "
                "`python -m redblackgraph_gb300.build` (nvcc, sm_103a)")
        lib = ctypes.CDLL(str(p))
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols():
    return [name for name, _, _ in SIGNATURES]


def dtype_code(dtype) -> int:
    try:
        return DTYPE_CODE[np.dtype(dtype)]
    except KeyError:
        raise TypeError(f"unsupported dtype {dtype}: AVOS kernels take 8/16/32/64-bit integers")


def check(rc: int, what: str) -> None:
    """Map a non-result status (argument / CUDA / memory errors) to a Python exception."""
    if rc == RBG_OK:
        return
    if rc == RBG_ERR_INVALID:
        raise ValueError(f"{what}: invalid argument")
    if rc == RBG_ERR_NOMEM:
        raise MemoryError(f"{what}: workspace too small or device memory budget exceeded")
    if rc == RBG_ERR_CUDA:
        raise RuntimeError(f"{what}: CUDA error")
    if rc == RBG_ERR_CAPACITY:
        raise RuntimeError(f"{what}: fixed-capacity buffer exceeded")
    if rc == RBG_ERR_TIMEOUT:
        raise TimeoutError(f"{what}: bounded device wait timed out")
    raise RuntimeError(f"{what}: status {rc}")
