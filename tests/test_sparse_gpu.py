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


def _squaring_diameter(P):
    """The reference's transitive_closure_gpu diameter (gpu/transitive_closure.py:52-72): the
    number of squarings R <- R (+) R^2 that change R, or floor(log2) of the largest |value| > 1 of
    the result when that is larger.  The squarings run on the oracle's CSR product; the sum keeps
    the smaller |value| per cell (R's on a tie)."""
    R = sorted_csr(sp.csr_matrix(P, dtype=np.int64))
    changing = 0
    for t in range(64):
        S, _ = O.rb_matmul_csr(R, R)
        S = sorted_csr(sp.csr_matrix(S, dtype=np.int64))
        Rd, Sd = R.toarray(), S.toarray()
        take = (Rd == 0) | ((Sd != 0) & (np.abs(Sd) < np.abs(Rd)))
        N = sorted_csr(sp.csr_matrix(np.where(take, Sd, Rd)))
        if same(N, R):
            break
        R, changing = N, t + 1
    a = np.abs(R.data)
    a = a[a > 1]
    return max(changing, int(np.floor(np.log2(a.max())))) if a.size else changing


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
    assert diam == _squaring_diameter(P)
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


def _star(parents: int, grand: bool):
    """Vertex 0 with `parents` parents (values 2/3), each with one parent of its own when `grand`:
    row 0 of the closure holds 1 + parents (+ parents) columns."""
    n = 1 + parents * (2 if grand else 1)
    r, c, v = [], [], []
    for i in range(n):
        r.append(i); c.append(i); v.append(-1 if i % 2 else 1)
    for i in range(1, parents + 1):
        r.append(0); c.append(i); v.append(2 + (i & 1))
        if grand:
            r.append(i); c.append(parents + i); v.append(3 - (i & 1))
    return sp.csr_matrix((np.array(v, dtype=np.int32), (np.array(r), np.array(c))), shape=(n, n))


def test_dag_levels_vs_oracle(native):
    """The level-parallel DAG closure (rbg_dag_closure) on permuted pedigree forests against the
    oracle's parents-first closure: entries and the candidate-maximum diameter."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    for seed, n, gens in ((5, 400, 10), (6, 900, 14), (7, 64, 3)):
        A = synth.forest(n, gens, seed, family=50, reach=3, dtype=np.int32)
        p = np.random.default_rng(seed).permutation(n)
        A = sp.csr_matrix(A[p][:, p])
        W, d = O.dag_closure(A)
        r = transitive_closure_dag_sparse(A)
        assert same(r.W, W) and r.diameter == d, seed


def test_dag_block_tier_pool_retry_and_levels(native):
    """Rows past the warp table (256 columns) go to the block tier; a pool too small is grown
    and the call repeated; the level count is the longest parent chain + 1."""
    import torch
    from redblackgraph_gb300.dag import dag_closure_device
    from redblackgraph_gb300.spgemm import DeviceCSR
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    A = _star(300, True)
    W, d = O.dag_closure(A)
    assert sp.csr_matrix(W)[0].nnz == 601
    r = transitive_closure_dag_sparse(A)
    assert same(r.W, W) and r.diameter == d
    C, mx, levels = dag_closure_device(DeviceCSR.from_scipy(A, dtype=np.int32, device="cuda"), pool_factor=0)
    torch.cuda.synchronize()
    assert same(C.to_scipy(), W) and levels == 3 and mx.bit_length() - 1 == d


def test_dag_row_too_wide_takes_squaring(native):
    """A row with more than 8192 columns is past the block table: RowTooWide from the level
    closure, and transitive_closure_dag_sparse answers by squaring with the same result."""
    from redblackgraph_gb300.dag import RowTooWide, dag_closure_device
    from redblackgraph_gb300.spgemm import DeviceCSR
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    A = _star(9000, False)
    with pytest.raises(RowTooWide):
        dag_closure_device(DeviceCSR.from_scipy(A, dtype=np.int32, device="cuda"))
    W, d = O.dag_closure(A)
    r = transitive_closure_dag_sparse(A)
    assert same(r.W, W) and r.diameter == d


def test_dag_cycle_below_a_dag(native):
    """Vertices under a cycle are never placed in a level: CycleError, also from the gpu module."""
    from redblackgraph_gb300.gpu import CSRMatrixGPU, transitive_closure_dag_gpu
    from redblackgraph_gb300.sparse import CycleError, transitive_closure_dag_sparse
    D = np.diag(np.array([-1, 1, -1, 1, -1], dtype=np.int32))
    D[0, 1] = 2; D[1, 2] = 3; D[2, 1] = 2; D[3, 4] = 3
    A = sp.csr_matrix(D)
    with pytest.raises(CycleError):
        transitive_closure_dag_sparse(A)
    with pytest.raises(CycleError):
        transitive_closure_dag_gpu(CSRMatrixGPU.from_cpu(A))


def test_dag_explicit_zeros_and_deep_rows(native):
    """Stored zeros stay in the closure (a zero product adds nothing), rows of 33-256 candidates
    take the merge of sorted runs; both against the oracle's parents-first closure."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    A = sp.lil_matrix(synth.forest(1500, 20, 11, family=40, reach=3, dtype=np.int32))
    n = A.shape[0]
    rng = np.random.default_rng(3)
    roots = [v for v in range(n) if A[v].nnz == 1]
    for v in rng.choice(n, size=40, replace=False):
        w = int(rng.choice(roots))
        if w != v and A[v, w] == 0:
            A[v, w] = 1          # placeholder, set to an explicit zero below
    A = sp.csr_matrix(A)
    A.data[A.data == 1] = np.where(A.indices[A.data == 1] == np.repeat(np.arange(n), np.diff(A.indptr))[A.data == 1],
                                   1, 0)
    assert (A.data == 0).sum() > 0
    W, d = O.dag_closure(A)
    r = transitive_closure_dag_sparse(A)
    assert same(r.W, W) and r.diameter == d
    assert (sp.csr_matrix(W).data == 0).sum() > 0
    lens = np.diff(sp.csr_matrix(W).indptr)
    assert lens.max() > 32


def test_dag_closure_tiny(native):
    """One vertex, and a graph of isolated vertices: the closure is the input."""
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    for M in (np.array([[1]]), np.diag([-1, 1, 1, -1])):
        A = sp.csr_matrix(M.astype(np.int32))
        r = transitive_closure_dag_sparse(A)
        assert same(r.W, A) and r.diameter == 0


def test_csr_diff_matches_host(native):
    """rbg_csr_diff: the entries of X absent from Y or holding another value there, for mixed
    storage types (an int32 squaring output against its int64 input)."""
    from redblackgraph_gb300.spgemm import DeviceCSR, csr_diff
    rng = np.random.default_rng(8)
    for xdt, ydt in ((np.int32, np.int32), (np.int32, np.int64), (np.int64, np.uint32)):
        Y = sp.random(700, 500, density=0.02, random_state=5, format="csr")
        Y.data = rng.integers(2, 60, size=Y.nnz).astype(np.float64)
        X = Y.copy()
        X.data[rng.random(X.nnz) < 0.1] += 1                      # changed values
        extra = sp.random(700, 500, density=0.01, random_state=6, format="csr")
        extra.data = rng.integers(2, 60, size=extra.nnz).astype(np.float64)
        X = (X + extra.multiply(Y == 0)).tocsr()                  # new entries
        X = sorted_csr(X.astype(xdt))
        Y = sorted_csr(Y.astype(ydt))
        Z = csr_diff(DeviceCSR.from_scipy(X), DeviceCSR.from_scipy(Y)).to_scipy()
        Xd, Yd = X.toarray().astype(np.int64), Y.toarray().astype(np.int64)
        exp = sp.csr_matrix(np.where((Xd != 0) & ((Yd == 0) | (Yd != Xd)), Xd, 0))
        assert Z.dtype == np.dtype(xdt)
        assert same(Z.astype(np.int64), exp.astype(np.int64))


@pytest.mark.parametrize("sem,upper", [(0, False), (1, False), (1, True)])
def test_semi_naive_squaring_equals_full_squaring(native, sem, upper):
    """Every step of the semi-naive loop (R (+) D R (+) R D when the last step changed at most
    half of R) equals the full step R (+) R^2, on a forest numbered oldest first and on the same
    forest renumbered at random; the number of changing steps is the full loop's."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.spgemm import DeviceCSR, spgemm, squaring_closure
    A = synth.forest(3000, 14, 6, family=60, reach=3, dtype=np.int32)
    p = np.random.default_rng(4).permutation(A.shape[0])
    mats = (A.T, sp.triu(sp.csr_matrix(A[p][:, p]))) if upper else (A, sp.csr_matrix(A[p][:, p]))
    for M in mats:
        M = sorted_csr(M)
        R = DeviceCSR.from_scipy(M)
        full = []
        for _ in range(64):
            Rn, _, _ = spgemm(R, R, R=R, upper=upper, sem=sem)
            full.append(Rn.to_scipy())
            if Rn.equal(R):
                break
            R = Rn
        forms = []
        for t in range(1, len(full) + 1):
            steps = []
            Rs, changed = squaring_closure(DeviceCSR.from_scipy(M), max_iterations=t, sem=sem, upper=upper,
                                           on_step=lambda rc, fl: None, steps=steps, seminaive=True)
            assert same(Rs.to_scipy(), full[t - 1]), t
            forms = [s[0] for s in steps]
        assert changed == len(full) - 1
        assert "semi-naive" in forms                               # the hybrid used both forms


def test_seminaive_operands_form_both_products(native):
    """[D R] [R ; D] equals D R (+) R D (each product on its own, then merged), values and
    pattern; the operands' shapes are n x 2n and 2n x n."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.spgemm import DeviceCSR, merge_minabs, seminaive_operands, spgemm, SEM_CY32
    A = synth.forest(2000, 12, 9, family=50, reach=3, dtype=np.int32)
    R = DeviceCSR.from_scipy(A)
    R1, _, _ = spgemm(R, R, R=R, sem=SEM_CY32)
    R2, _, _ = spgemm(R1, R1, R=R1, sem=SEM_CY32)
    from redblackgraph_gb300.spgemm import csr_diff
    D = csr_diff(R2, R1)
    assert D.nnz > 0
    A2, B2 = seminaive_operands(D, R2)
    assert A2.shape == (2000, 4000) and B2.shape == (4000, 2000) and A2.nnz == B2.nnz == D.nnz + R2.nnz
    got, _, _ = spgemm(A2, B2, sem=SEM_CY32)
    P1, _, _ = spgemm(D, R2, sem=SEM_CY32)
    P2, _, _ = spgemm(R2, D, sem=SEM_CY32)
    exp = merge_minabs(P1, P2)
    assert same(got.to_scipy(), exp.to_scipy())
