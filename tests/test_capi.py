"""The C-ABI library loads and exports every entry point include/rbg_gb300.h declares.
CPU only: no compute call is made."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = "\n".join(p.read_text() for p in (ROOT / "include").glob("*.h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rbg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    syms = declared_symbols()
    assert len(syms) >= 6
    for s in syms:
        assert hasattr(native, s), s


def test_python_binding_covers_header(native):
    from redblackgraph_gb300 import _lib
    assert sorted(_lib.exported_symbols()) == declared_symbols()


def test_workspace_queries_without_gpu(native):
    from redblackgraph_gb300 import _lib
    n = ctypes.c_int64(0)
    assert native.rbg_fw_dense_workspace_bytes(4, 1000, 0, ctypes.byref(n)) == 0
    assert n.value >= 1024 * 1024 * 4
    assert native.rbg_fw_dense_workspace_bytes(99, 10, 0, ctypes.byref(n)) == _lib.RBG_ERR_INVALID
    assert native.rbg_version() > 0


def test_batch_workspace_sizes_are_stable(native):
    """rbg_fw_batch_workspace_bytes (host only) gives the same size for a layout asked again (the
    answer is cached per layout), distinguishes layouts, dtypes and the triangular mode, and grows
    with the batch."""
    import numpy as np

    def size(sizes, dtype=4, mode=0):
        s = np.ascontiguousarray(sizes, dtype=np.int64)
        b = ctypes.c_int64(0)
        assert native.rbg_fw_batch_workspace_bytes(dtype, s.size, s.ctypes.data, mode, ctypes.byref(b)) == 0
        return b.value

    a = [16, 300, 4096, 17, 1]
    first = size(a)
    assert all(size(a) == first for _ in range(3))
    assert size(a + [200]) > first
    assert size(a, dtype=6) != first                 # 64-bit storage: other lane buffers
    for k in range(6):                               # more layouts than the cache holds
        size([64 * (k + 1)] * 3)
    assert size(a) == first
    assert size([]) >= 0
    bad = np.array([-1], np.int64)
    out = ctypes.c_int64(0)
    assert native.rbg_fw_batch_workspace_bytes(4, 1, bad.ctypes.data, 0, ctypes.byref(out)) != 0


def test_cc_dag_classify_refuses_malformed_components(native):
    """rbg_cc_dag_classify checks its arguments before anything reaches the GPU: a graph of n > 0
    vertices without components, more components than vertices, or a missing buffer is
    RBG_ERR_INVALID (every call here fails that check, so nothing is launched)."""
    from redblackgraph_gb300 import _lib
    buf = ctypes.create_string_buffer(4096)
    p = ctypes.addressof(buf)
    edges = ctypes.c_int64(-1)

    def classify(n, ncomp, start=p, flags=p):
        return native.rbg_cc_dag_classify(n, p, p, p, p, start, ncomp, p, 4096, flags, p, p,
                                          ctypes.byref(edges), None)

    assert classify(5, 0) == _lib.RBG_ERR_INVALID
    assert classify(5, 6) == _lib.RBG_ERR_INVALID
    assert classify(-1, 0) == _lib.RBG_ERR_INVALID
    assert classify(5, 2, start=None) == _lib.RBG_ERR_INVALID
    assert classify(5, 2, flags=None) == _lib.RBG_ERR_INVALID
    assert edges.value == -1                         # refused before any output was touched
