"""Sparse AVOS product and squaring closures on the GPU against the oracle and the reference's
golden answers (bit-exact)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def sorted_csr(m):
    m = sp.csr_matrix(m, copy=True)
    m.sort_indices()
    return m


def same(a, b):
    a, b = sorted_csr(a), sorted_csr(b)
    return (a.shape == b.shape and a.nnz == b.nnz and (a.indptr == b.indptr).all()
            and (a.indices == b.indices).all() and (a.data == b.data).all())


def test_golden_rb_matrix_products(native, golden):
    from redblackgraph_gb300.sparse import rb_matrix
    arrays, index = golden
    for rec in index["spgemm"]:
        k, n = rec["key"], rec["n"]
        M = rb_matrix(sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]),
                                    shape=(n, n)))
        C = M @ M
        E = sp.csr_matrix((arrays[k + "_C_data"], arrays[k + "_C_indices"], arrays[k + "_C_indptr"]),
                          shape=(n, n))
        assert same(C, E), rec
        assert C.dtype == M.dtype


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint32, np.uint64, np.int16])
def test_rb_matrix_vs_oracle(native, dtype):
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import rb_matrix
    A = synth.forest(5000, 12, 3, family=48, reach=3, dtype=np.int64)
    W = A.astype(dtype)
    if np.dtype(dtype).kind == "u":
        W.data[A.data == -1] = np.iinfo(dtype).max
    M = rb_matrix(W)
    R = M
    for _ in range(3):                      # products of growing density
        C = R @ M
        Co, _ = O.rb_matmul_csr(R, M)
        assert same(C, Co)
        R = rb_matrix(C)


def test_block_and_dense_rows(native):
    """Rows beyond the warp (1024) and block (8192) candidate capacities."""
    from redblackgraph_gb300.sparse import rb_matrix
    rng = np.random.default_rng(5)
    n = 3000
    A = sp.random(n, n, density=0.02, random_state=6, format="csr")
    A.data = rng.integers(2, 9, size=A.nnz).astype(np.float64)
    A = A.astype(np.int64)
    A.setdiag(1)
    A = A.tocsr()
    A[7, :] = 0
    A[7, : n // 2] = 3                      # one row touching ~half of the rows of B
    A.eliminate_zeros()
    A = A.tocsr()
    M = rb_matrix(A)
    C = M @ M
    Co, fl = O.rb_matmul_csr(A, A)
    assert same(C, Co)


def test_gpu_module_spgemm_and_mask(native):
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.gpu import CSRMatrixGPU, spgemm, spgemm_upper_triangular
    A = synth.forest(4000, 10, 8, family=40, reach=2, dtype=np.int32)
    U = sp.csr_matrix(A.T)                  # upper triangular pedigree
    G = CSRMatrixGPU.from_cpu(U)
    assert G.triangular
    C = spgemm(G)                           # masked j >= i by default for a triangular self product
    Co, _ = O.rb_matmul_csr(U.astype(np.int64), U.astype(np.int64))
    assert same(C.to_cpu(), sp.triu(Co).astype(np.int32))
    C2 = spgemm_upper_triangular(G)
    assert same(C2.to_cpu(), C.to_cpu())
    D = spgemm(G, G, upper_triangular=False)
    assert same(D.to_cpu(), Co.astype(np.int32))
    assert (G @ G).nnz == C.nnz


def _dense_closure(A):
    W, d, st, _ = O.warshall(np.asarray(A.toarray(), dtype=np.int64))
    assert st == 0
    return sp.csr_matrix(W.astype(np.int32))


def test_squaring_closures_match_dense_oracle(native):
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import transitive_closure_squaring, transitive_closure_dag_sparse
    from redblackgraph_gb300.gpu import CSRMatrixGPU, transitive_closure_gpu, transitive_closure_dag_gpu
    A = synth.forest(600, 12, 4, family=60, reach=3, dtype=np.int32)
    E = _dense_closure(A)
    r = transitive_closure_squaring(A)      # lower triangular: the DAG closure
    assert same(r.W, E)
    assert r.diameter == O.dag_closure(A)[1]   # the DAG closure's candidate-maximum diameter
    r2 = transitive_closure_dag_sparse(A)
    assert same(r2.W, E) and r2.diameter == r.diameter
    # a DAG that is not triangular: permute the vertices
    p = np.random.default_rng(1).permutation(A.shape[0])
    P = sp.csr_matrix(A[p][:, p])
    rp = transitive_closure_squaring(P)
    Ep = _dense_closure(P)
    assert same(rp.W, Ep)
    assert rp.diameter == int(np.floor(np.log2(np.abs(Ep.data).max())))
    G = CSRMatrixGPU.from_cpu(P)
    R, diam = transitive_closure_gpu(G)
    assert same(R.to_cpu(), Ep)
    Rd, dd = transitive_closure_dag_gpu(G)
    assert same(Rd.to_cpu(), Ep) and dd == int(np.floor(np.log2(np.abs(Ep.data).max())))


def test_cycle_raises_in_dag_closure(native):
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse, CycleError
    A = sp.csr_matrix(np.array([[-1, 2, 0], [0, 1, 3], [2, 0, -1]], dtype=np.int32))
    with pytest.raises(CycleError):
        transitive_closure_dag_sparse(A)


def test_sparse_avos_sum_gpu_matches_rule(native):
    from redblackgraph_gb300.gpu import CSRMatrixGPU
    from redblackgraph_gb300.gpu.transitive_closure import sparse_avos_sum_gpu
    rng = np.random.default_rng(2)
    X = sp.random(300, 300, density=0.05, random_state=3, format="csr")
    Y = sp.random(300, 300, density=0.05, random_state=4, format="csr")
    X.data = rng.choice([-1, 1, 2, 3, -5, 9], size=X.nnz).astype(np.float64)
    Y.data = rng.choice([-1, 1, 2, 3, 5, -9, 4], size=Y.nnz).astype(np.float64)
    X, Y = X.astype(np.int32), Y.astype(np.int32)
    Z = sparse_avos_sum_gpu(CSRMatrixGPU.from_cpu(X), CSRMatrixGPU.from_cpu(Y)).to_cpu().toarray()
    xd, yd = X.toarray(), Y.toarray()
    exp = np.where(xd == 0, yd, np.where(yd == 0, xd, np.where(np.abs(yd) < np.abs(xd), yd, xd)))
    assert (Z == exp).all()


def test_golden_dijkstra_method(native, golden):
    from redblackgraph_gb300.sparse import transitive_closure
    arrays, index = golden
    for rec in index["dijkstra"]:
        A = arrays[rec["key"] + "_in"]
        r = transitive_closure(sp.csr_matrix(A), method="D")
        assert (np.asarray(r.W) == arrays[rec["key"] + "_W"]).all()
        assert r.diameter == rec["diameter"]


def test_golden_dag_closure(native, golden):
    """transitive_closure_dag_sparse against the reference: the closure and its diameter, which
    counts candidates that lose the (+) (in two of these forests it exceeds MSB of the largest
    final value)."""
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse, transitive_closure_squaring
    arrays, index = golden
    for rec in index["dag"]:
        k, n = rec["key"], rec["n"]
        A = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]), shape=(n, n))
        E = sp.csr_matrix((arrays[k + "_W_data"], arrays[k + "_W_indices"], arrays[k + "_W_indptr"]), shape=(n, n))
        for fn in (transitive_closure_dag_sparse, transitive_closure_squaring):
            r = fn(A)
            assert same(r.W, E), (k, fn.__name__)
            assert r.diameter == rec["diameter"], (k, fn.__name__, r.diameter, rec["diameter"])
