"""The dense closure entry point that allocates nothing (rbg_fw_dense_noalloc).

It exists for callers that cannot call cudaMalloc -- code that runs where allocating is
forbidden or unsafe, or a host program that owns only its input and output buffers.  Its
scratch lives in a fixed array inside the library, shared by every call, so these tests check
that its results equal the workspace entry point's (bit-exact integers) on two calls in a row
with different inputs, and that a size beyond the array is refused.  This file is named to be
collected last; it must pass alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close_with_workspace(L, _lib, d, out):
    import torch
    from redblackgraph_gb300.device import numpy_dtype, stream_handle
    n = d.shape[0]
    code = _lib.dtype_code(numpy_dtype(d.dtype))
    nbytes = ctypes.c_int64(0)
    assert L.rbg_fw_dense_workspace_bytes(code, n, 0, ctypes.byref(nbytes)) == _lib.RBG_OK
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=d.device)
    res = _lib.RbgResult()
    rc = L.rbg_fw_dense(code, n, d.data_ptr(), n, out.data_ptr(), n, 0, ws.data_ptr(), ws.numel(),
                        ctypes.byref(res), stream_handle())
    assert rc == _lib.RBG_OK
    return res


def _close_without_workspace(L, _lib, d, out):
    from redblackgraph_gb300.device import numpy_dtype, stream_handle
    n = d.shape[0]
    res = _lib.RbgResult()
    rc = L.rbg_fw_dense_noalloc(_lib.dtype_code(numpy_dtype(d.dtype)), n, d.data_ptr(), n,
                                out.data_ptr(), n, 0, ctypes.byref(res), stream_handle())
    assert rc == _lib.RBG_OK
    return res


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(native):
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.device import to_device, to_host
    L = native
    cases = [(700, 14, 11, np.int32), (_lib.NOALLOC_MAX_N, 16, 12, np.int64)]
    for n, gens, seed, dtype in cases:          # two calls in a row, different inputs
        A = synth.pedigree(n, gens, seed, dtype=dtype)
        d = to_device(A)
        ref_out = torch.empty_like(d)
        ref = _close_with_workspace(L, _lib, d, ref_out)
        out = torch.full_like(d, 7)             # stale contents must not leak into the result
        res = _close_without_workspace(L, _lib, d, out)
        torch.cuda.synchronize()
        assert res.status == ref.status == _lib.RBG_OK
        assert res.diameter == ref.diameter and res.path == ref.path
        assert (to_host(out) == to_host(ref_out)).all()
        assert (to_host(d) == A).all()          # the input is left untouched


def _wide_int64():
    """A pedigree whose last vertex with parents reaches its first parent by an edge value past
    2^31 (closure values past bit 31): the blocked kernels with 64-bit lanes."""
    from redblackgraph_gb300 import synth
    A = synth.pedigree(200, 10, 9, dtype=np.int64)
    i = int(np.nonzero((A > 1).any(axis=1))[0][-1])
    p = int(np.nonzero(A[i] > 1)[0][0])
    A[i, p] <<= 32
    return A


def _unclean_int32(n):
    """Random upper-triangular values 0..3 (value 1 off the diagonal): the exact kernel."""
    rs = np.random.RandomState(5)
    A = np.triu(rs.randint(0, 4, size=(n, n)), k=1)
    np.fill_diagonal(A, rs.choice([-1, 1], size=n))
    return A.astype(np.int32)


PATH_CASES = ["dag_int32", "blocked64", "exact", "dag_int64"]


@pytest.mark.parametrize("case", PATH_CASES)
def test_noalloc_every_path_inside_its_array(native, case):
    """The fixed array also holds the scratch of the other paths a closure can take: the DAG
    path, the blocked kernels with 64-bit lanes and the exact sequential-order kernel (with its
    status block).  Each case runs twice in a row, takes its path and equals the oracle's
    sequential loop (values, diameter, status)."""
    import torch
    from oracle import oracle as O
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.device import to_device, to_host
    L = native
    A, path = {"dag_int32": lambda: (synth.pedigree(900, 15, 3, dtype=np.int32), _lib.PATH_DAG),
               "blocked64": lambda: (_wide_int64(), _lib.PATH_BLOCKED64),
               "exact": lambda: (_unclean_int32(300), _lib.PATH_EXACT),
               "dag_int64": lambda: (synth.pedigree(_lib.NOALLOC_MAX_N, 20, 4, dtype=np.int64), _lib.PATH_DAG)}[case]()
    Wo, do, so, info = O.warshall(A)
    d = to_device(A)
    for _ in range(2):
        out = torch.full_like(d, 5)
        res = _close_without_workspace(L, _lib, d, out)
        torch.cuda.synchronize()
        assert res.path == path
        assert (res.status, res.diameter) == (so, do)
        if so == _lib.RBG_OK:
            assert (to_host(out) == Wo).all()
        else:
            assert (res.k, res.i, res.j) == tuple(info[2:5])
        assert (to_host(d) == A).all()


def test_noalloc_refuses_sizes_beyond_its_array(native):
    import torch
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.device import stream_handle
    n = _lib.NOALLOC_MAX_N + 1
    d = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    res = _lib.RbgResult()
    rc = native.rbg_fw_dense_noalloc(4, n, d.data_ptr(), n, d.data_ptr(), n, 0, ctypes.byref(res),
                                     stream_handle())
    assert rc == _lib.RBG_ERR_CAPACITY
