"""Dense closure and dense AVOS product on the GPU against the oracle and the reference's
golden answers.  Integer work: every comparison is bit-exact (W, diameter, exception)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EXC = {0: None, 1: OverflowError, 2: ValueError}
NAMES = {None: None, "OverflowError": OverflowError, "ValueError": ValueError,
         "CycleError": ValueError}


def gpu_close(A, mode=0):
    import torch
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    d = to_device(np.ascontiguousarray(A))
    out, res = fw_dense(d, mode=mode)
    torch.cuda.synchronize()
    return to_host(out), res


def test_golden_warshall_through_drop_in(native, golden):
    import redblackgraph_gb300 as rbg
    arrays, index = golden
    for rec in index["warshall"]:
        A = arrays[rec["key"] + "_in"]
        exp = NAMES[rec["exception"]]
        if exp is None:
            res = rbg.array(A).transitive_closure()
            assert isinstance(res.W, rbg.array)
            assert (np.asarray(res.W) == arrays[rec["key"] + "_W"]).all(), rec
            assert int(res.diameter) == rec["diameter"], rec
        else:
            with pytest.raises(exp):
                rbg.array(A).transitive_closure()


def test_golden_cython_floyd_warshall(native, golden):
    from redblackgraph_gb300.sparse import floyd_warshall, CycleError
    arrays, index = golden
    for rec in index["cython"]:
        A = arrays[rec["key"] + "_in"]
        if rec["exception"] == "CycleError":
            with pytest.raises(CycleError) as ei:
                floyd_warshall(A, assume_upper_triangular=rec["triangular"])
            assert ei.value.vertex == rec["vertex"]
        else:
            W, d = floyd_warshall(A, assume_upper_triangular=rec["triangular"])
            assert (np.asarray(W) == arrays[rec["key"] + ("_cyT" if rec["triangular"] else "_cy")]).all()
            assert d == rec["diameter"]


@pytest.mark.parametrize("n,gens,dtype", [
    (64, 6, np.int32), (127, 8, np.int32), (128, 9, np.int64), (129, 9, np.uint32),
    (200, 12, np.int16), (511, 12, np.int32), (512, 12, np.int32), (700, 20, np.int64),
    (1024, 14, np.int32), (300, 40, np.int64), (257, 30, np.uint64), (90, 8, np.uint8),
])
def test_seeded_pedigrees_vs_oracle(native, n, gens, dtype):
    from redblackgraph_gb300 import synth, _lib
    A = synth.pedigree(n, gens, seed=n * 31 + gens, dtype=dtype)
    Wo, do, so, info = O.warshall(A)
    W, res = gpu_close(A)
    assert res.status == so
    if so == 0:
        assert (W == Wo).all()
        assert res.diameter == do


@pytest.mark.parametrize("seed", [42, 123, 456, 7])
def test_unclean_random_triu_exact_path(native, seed):
    from redblackgraph_gb300 import _lib
    rs = np.random.RandomState(seed)
    n = 70
    A = np.triu(rs.randint(0, 4, size=(n, n)), k=1)
    np.fill_diagonal(A, rs.choice([-1, 1], size=n))
    for dt in (np.int32, np.int64):
        Wo, do, so, _ = O.warshall(A.astype(dt))
        W, res = gpu_close(A.astype(dt))
        assert res.path == _lib.PATH_EXACT
        assert res.status == so and (so != 0 or ((W == Wo).all() and res.diameter == do))
        Wc, dc, sc, _ = O.fw_cython(A.astype(np.int32))
        W2, r2 = gpu_close(A.astype(np.int32), mode=_lib.MODE_CYTHON)
        assert r2.status == sc and (W2 == Wc).all() and r2.diameter == dc


def test_forced_exact_equals_blocked(native):
    """The same pedigree on the DAG path (the default for a matrix numbered oldest first), on
    the blocked kernels (RBG_MODE_NO_DAG) and on the exact sequential-order kernel."""
    from redblackgraph_gb300 import synth, _lib
    A = synth.pedigree(333, 15, 5, dtype=np.int32)
    W0, r0 = gpu_close(A)
    W1, r1 = gpu_close(A, mode=_lib.MODE_NO_DAG)
    W2, r2 = gpu_close(A, mode=_lib.MODE_FORCE_EXACT)
    assert r0.path == _lib.PATH_DAG and r1.path == _lib.PATH_BLOCKED32 and r2.path == _lib.PATH_EXACT
    assert (W0 == W1).all() and (W1 == W2).all() and r0.diameter == r1.diameter == r2.diameter


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
@pytest.mark.parametrize("above", [False, True])
def test_single_matrix_dag_path(native, dtype, above):
    """rbg_fw_dense takes the DAG path for an int32 or int64 matrix numbered in a topological
    order (entries below the diagonal, or above it), out of place, in place and into rows with a
    longer stride; values, diameter and status are the oracle's sequential loop's."""
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    for n, gens in ((1, 1), (7, 3), (300, 12), (1025, 15), (2000, 30)):
        A = synth.pedigree(n, gens, seed=n + 3, dtype=dtype)
        if above:
            A = A[::-1, ::-1].copy()
        Wo, do, so, _ = O.warshall(A)
        assert so == 0
        W, res = gpu_close(A)
        assert res.path == _lib.PATH_DAG and res.status == 0, (n, res.path)
        assert (W == Wo).all() and res.diameter == do
        d = to_device(A)
        _, ri = fw_dense(d, out=d)                        # in place
        assert ri.path == _lib.PATH_DAG and (to_host(d) == Wo).all() and ri.diameter == do
        big = torch.full((n, n + 5), 77, dtype=d.dtype, device=d.device)
        view = big[:, 2:n + 2]                            # rows 16-byte misaligned, stride n + 5
        _, rv = fw_dense(to_device(A), out=view)
        torch.cuda.synchronize()
        hb = big.cpu().numpy()
        assert rv.path == _lib.PATH_DAG and (hb[:, 2:n + 2] == Wo).all()
        assert (hb[:, :2] == 77).all() and (hb[:, n + 2:] == 77).all()   # nothing outside the view


def test_single_matrix_dag_path_graph_mode(native):
    """RBG_MODE_GRAPH on a single matrix: recorded once (level loop as a device-driven while
    node), replayed on later calls; every call equals the direct launches and the oracle, also
    after the input changes in place."""
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    A = synth.pedigree(1500, 25, 4, dtype=np.int64)
    Wo, do, so, _ = O.warshall(A)
    d = to_device(A)
    out = torch.empty_like(d)
    for _ in range(3):
        _, r = fw_dense(d, out=out, mode=_lib.MODE_GRAPH)
        torch.cuda.synchronize()
        assert r.path == _lib.PATH_DAG and (to_host(out) == Wo).all() and r.diameter == do
    B = synth.pedigree(1500, 25, 5, dtype=np.int64)
    Wb, db, _, _ = O.warshall(B)
    d.copy_(to_device(B))
    _, r = fw_dense(d, out=out, mode=_lib.MODE_GRAPH)
    torch.cuda.synchronize()
    assert r.path == _lib.PATH_DAG and (to_host(out) == Wb).all() and r.diameter == db


def test_wide_lanes_int64(native):
    """64-bit values beyond 2^31: the 32-bit lane attempt hands over to 64-bit lanes."""
    from redblackgraph_gb300 import synth, _lib
    A = synth.pedigree(200, 10, 9, dtype=np.int64)
    # every parent edge spans 9 generations: closure values pass 2^31
    A = np.where((A > 1), A.astype(np.int64) << 8, A)
    Wo, do, so, _ = O.warshall(A)
    assert Wo.max() >= 2**31
    W, res = gpu_close(A)
    assert so == 0 and res.status == 0
    assert res.path == _lib.PATH_BLOCKED64
    assert (W == Wo).all() and res.diameter == do


def test_risk_reruns_exactly(native):
    """An int32 chain deep enough to reach the top bit leaves the blocked path."""
    from redblackgraph_gb300 import _lib
    n = 34
    A = np.zeros((n, n), np.int64)
    np.fill_diagonal(A, 1)
    for i in range(n - 1):
        A[i + 1, i] = 2
    for dt in (np.int32, np.uint32):
        Wo, do, so, _ = O.warshall(A.astype(dt))
        W, res = gpu_close(A.astype(dt))
        assert res.path == _lib.PATH_EXACT
        assert res.status == so


def test_cycles_and_last_error(native):
    from redblackgraph_gb300 import synth, _lib
    A = synth.pedigree(400, 10, 17, dtype=np.int32)
    C, _, _, _ = O.warshall(A)
    v, u = max(zip(*np.nonzero(np.tril(C, -1))), key=lambda t: t[0] - t[1])
    A[u, v] = 2   # u is an ancestor of v; making v a parent of u closes a cycle
    Wo, do, so, info = O.warshall(A)
    W, res = gpu_close(A)
    assert so == _lib.RBG_ERR_CYCLE and res.status == so
    assert (res.k, res.i, res.j) == tuple(info[2:5])
    Wc, dc, sc, ic = O.fw_cython(A)
    W2, r2 = gpu_close(A, mode=_lib.MODE_CYTHON)
    assert r2.status == sc == _lib.RBG_ERR_CYCLE and r2.i == ic[2]


def test_in_place_and_triangular(native):
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    A = synth.pedigree(300, 12, 2, dtype=np.int32)
    d = to_device(A)
    out, res = fw_dense(d, out=d)
    Wo, do, so, _ = O.warshall(A)
    assert out.data_ptr() == d.data_ptr() and (to_host(out) == Wo).all() and res.diameter == do
    U = np.ascontiguousarray(A.T)
    U[5, 2] = 2   # a lower entry the triangular loop never reads
    Wt, dt_, st, _ = O.fw_cython(U, triangular=True)
    W2, r2 = gpu_close(U, mode=_lib.MODE_CYTHON | _lib.MODE_TRIANGULAR)
    assert r2.status == st == 0 and (W2 == Wt).all() and r2.diameter == dt_


def test_empty_and_tiny(native):
    import redblackgraph_gb300 as rbg
    for n in (1, 2, 3):
        A = np.eye(n, dtype=np.int32)
        r = rbg.array(A).transitive_closure()
        assert (np.asarray(r.W) == A).all() and r.diameter == 0
    W, d = rbg.warshall(np.zeros((0, 0), np.int32))
    assert W.shape == (0, 0)


def test_stacked_warshall(native):
    import redblackgraph_gb300 as rbg
    from redblackgraph_gb300 import synth
    As = np.stack([synth.pedigree(50, 6, s, dtype=np.int64) for s in range(3)])
    W, d = rbg.warshall(As)
    for b in range(3):
        Wo, do, _, _ = O.warshall(As[b])
        assert (W[b] == Wo).all() and d[b] == do


def test_golden_matmul(native, golden):
    import redblackgraph_gb300 as rbg
    arrays, index = golden
    for rec in index["matmul"]:
        A = arrays[rec["key"] + "_in"]
        C = rbg.array(A) @ rbg.array(A)
        assert (np.asarray(C) == arrays[rec["key"] + "_AA"]).all(), rec


@pytest.mark.parametrize("dtype", [np.int32, np.uint16, np.int64])
def test_matmul_vs_oracle(native, dtype):
    import redblackgraph_gb300 as rbg
    from redblackgraph_gb300 import synth
    A = synth.pedigree(150, 10, 4, dtype=dtype)
    W, _, _, _ = O.warshall(A)
    C, st, _ = O.matmul(W, A)
    G = rbg.array(W) @ rbg.array(A)
    assert st == 0 and (np.asarray(G) == C).all()
    v = A[:, 3].copy()
    assert (rbg.array(W) @ v == O.matmul(W, v.reshape(-1, 1))[0].reshape(-1)).all()


def test_matmul_overflow(native):
    import redblackgraph_gb300 as rbg
    a = rbg.array([[2**20]], dtype=np.int32)
    b = rbg.array([[2**20]], dtype=np.int32)
    with pytest.raises(OverflowError):
        a @ b


def test_scalar_tables_on_device(native, golden):
    from redblackgraph_gb300.elementwise import avos_product_array, avos_sum_array
    arrays, _ = golden
    r = np.arange(-1, 16)
    X, Y = np.meshgrid(r, r, indexing="ij")
    P = avos_product_array(X.astype(np.int64), Y.astype(np.int64))
    assert (P.astype(np.int64) == arrays["scalar_product_table"]).all()
    r2 = np.arange(-1, 4)
    X, Y = np.meshgrid(r2, r2, indexing="ij")
    assert (avos_sum_array(X, Y) == arrays["scalar_sum_table"]).all()


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_single_matrix_any_numbering_dag_path(native, dtype):
    """rbg_fw_dense on relabelled pedigrees (entries on both sides of the diagonal): the DAG path
    replays the loop in the given numbering; W and diameter equal the oracle's."""
    from redblackgraph_gb300 import synth, _lib
    rng = np.random.default_rng(5)
    for n in (5, 200, 1024, 1800):
        A = synth.pedigree(n, synth.generations_for(n), n + 9, dtype=dtype)
        p = rng.permutation(n)
        A = A[p][:, p].copy()
        Wo, do, so, _ = O.warshall(A)
        W, res = gpu_close(A)
        assert so == 0 and res.status == 0
        assert (W == Wo).all() and res.diameter == do
        assert res.path == _lib.PATH_DAG, (n, res.path)


def test_kernel_attributes_on_every_device(native):
    """Kernels with more than 48 KB of shared memory get their attribute on each device the
    process uses: a blocked closure, a DAG-path closure and a sparse product on device 1 after
    device 0, each equal to the oracle (needs two visible GPUs)."""
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    from redblackgraph_gb300.spgemm import DeviceCSR, spgemm
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    A = synth.pedigree(500, 12, 3, dtype=np.int32)
    Wo, do, so, _ = O.warshall(A)
    Po, _ = O.rb_matmul_csr(A, A)
    for dev in (0, 1):
        with torch.cuda.device(dev):
            d = to_device(A, torch.device("cuda", dev))
            for mode, path in ((_lib.MODE_NO_DAG, _lib.PATH_BLOCKED32), (0, _lib.PATH_DAG)):
                out, r = fw_dense(d, mode=mode)
                torch.cuda.synchronize(dev)
                assert r.path == path and (to_host(out) == Wo).all() and r.diameter == do
            M = DeviceCSR.from_scipy(A, device=torch.device("cuda", dev))
            P, rc, _ = spgemm(M, M)
            assert rc == 0 and (P.to_scipy() != Po).nnz == 0
