"""The CPU oracle against the reference's own answers (golden fixtures made by running the
reference, tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O

EXC = {0: None, 1: "OverflowError", 2: "ValueError"}


def test_product_table(golden):
    arrays, _ = golden
    exp = arrays["scalar_product_table"]
    r = range(-1, 16)
    got = np.array([[O.avos_product(x, y, np.int64)[0] for y in r] for x in r], dtype=np.uint64)
    assert (got.astype(np.int64) == exp).all()


def test_sum_table(golden):
    arrays, _ = golden
    exp = arrays["scalar_sum_table"]
    r = range(-1, 4)
    got = np.array([[O.avos_sum(x, y, np.int64) for y in r] for x in r])
    assert (got == exp).all()


def test_edge_and_overflow(golden):
    _, index = golden
    x, y, z = index["scalar"]["edge_product"]
    v, ev = O.avos_product(int(x), int(y), np.uint64)
    assert v == int(z) and ev == 0
    for x, y, exc in index["scalar"]["overflow"]:
        v, ev = O.avos_product(int(x), int(y), np.uint64)
        assert (ev & (O.EV_OVF_SIZE | O.EV_OVF_ONES)) != 0
        assert exc == "OverflowError"


def test_cython_scalar_matches_core_on_small_values():
    for x in range(-1, 40):
        for y in range(-1, 40):
            v, ev = O.avos_product(x, y, np.int32)
            assert O.cy_product(x, y) == np.int64(np.uint32(v).view(np.int32))
            assert O.cy_sum(x, y) == O.avos_sum(x, y, np.int32) or (x < -1 or y < -1)


def test_warshall_cases(golden):
    arrays, index = golden
    for rec in index["warshall"]:
        A = arrays[rec["key"] + "_in"]
        W, d, st, info = O.warshall(A)
        assert EXC[st] == rec["exception"], rec
        if rec["exception"] is None:
            assert (W == arrays[rec["key"] + "_W"]).all(), rec
            assert d == rec["diameter"], rec
        if rec.get("reference") == "hang":
            assert info[1] & O.EV_HANG


def test_cython_cases(golden):
    arrays, index = golden
    for rec in index["cython"]:
        A = arrays[rec["key"] + "_in"]
        W, d, st, info = O.fw_cython(A, triangular=rec["triangular"])
        if rec["exception"] == "CycleError":
            assert st == O.RBG_ERR_CYCLE and info[2] == rec["vertex"], rec
        else:
            assert st == 0
            assert (W == arrays[rec["key"] + ("_cyT" if rec["triangular"] else "_cy")]).all(), rec
            assert d == rec["diameter"], rec


def test_matmul_cases(golden):
    arrays, index = golden
    for rec in index["matmul"]:
        A = arrays[rec["key"] + "_in"]
        C, st, fl = O.matmul(A, A)
        assert EXC[st] == rec["exception"]
        if st == 0:
            assert (C == arrays[rec["key"] + "_AA"]).all(), rec


def test_spgemm_cases(golden):
    import scipy.sparse as sp
    arrays, index = golden
    for rec in index["spgemm"]:
        k = rec["key"]
        n = rec["n"]
        M = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]),
                          shape=(n, n))
        C, fl = O.rb_matmul_csr(M, M)
        C.sort_indices()
        assert (C.indptr == arrays[k + "_C_indptr"]).all()
        assert (C.indices == arrays[k + "_C_indices"]).all()
        assert (C.data == arrays[k + "_C_data"]).all()


def test_warshall_triangular_equals_full_on_upper():
    from redblackgraph_gb300 import synth
    A = synth.pedigree(60, 6, 3, dtype=np.int32).T.copy()   # upper triangular
    W1, d1, s1, _ = O.warshall(A)
    W2, d2, s2, _ = O.warshall(A, triangular=True)
    assert (W1 == W2).all() and d1 == d2 and s1 == s2 == 0


def test_oracle_component_wise_closure_vs_golden(golden):
    """The component split, per-component closure, merge and diameter rule against the
    reference's component_wise_closure on forests with shuffled vertices."""
    import scipy.sparse as sp
    arrays, index = golden
    for rec in index["components"]:
        k, n = rec["key"], rec["n"]
        A = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]), shape=(n, n))
        W, d, err = O.component_wise_closure(A, rec["method"], rec["threshold"])
        if "error" in rec:
            assert err is not None and rec["error"] == "CycleError"
            assert int(err[1][2]) == rec["vertex"]      # the reference reports the local vertex
            continue
        E = sp.csr_matrix((arrays[k + "_W_data"], arrays[k + "_W_indices"], arrays[k + "_W_indptr"]),
                          shape=(n, n))
        assert d == rec["diameter"], rec
        assert (W.indptr == E.indptr).all() and (W.indices == E.indices).all() and (W.data == E.data).all()


def test_oracle_relationship_vs_golden(golden):
    """Relationship lookups against the reference's calculate_relationship on closure rows
    (numpy rows: sums wrap in the rows' dtype, as numpy scalar arithmetic does)."""
    arrays, index = golden
    for rec in index["relationship"]:
        W = arrays[rec["key"] + "_W"]
        for u, v, ca, name in rec["pairs"]:
            assert O.calculate_relationship(W[u], W[v]) == (ca, name), (rec["key"], u, v)


def test_oracle_dag_closure_vs_golden(golden):
    """The DAG-closure restatement (closure and its candidate-maximum diameter) against the
    reference's transitive_closure_dag_sparse."""
    import scipy.sparse as sp
    arrays, index = golden
    for rec in index["dag"]:
        k, n = rec["key"], rec["n"]
        A = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]), shape=(n, n))
        E = sp.csr_matrix((arrays[k + "_W_data"], arrays[k + "_W_indices"], arrays[k + "_W_indptr"]), shape=(n, n))
        W, d = O.dag_closure(A)
        assert d == rec["diameter"]
        assert (W != E).nnz == 0


def test_oracle_relational_composition_vs_golden(golden):
    """The composition restatements (C core, every storage type; Cython, int32) against the
    reference's core and csgraph functions.  Where the reference's gufunc raised (or took the
    interpreter down raising from its loop), the oracle reports the error; where its MSB loop
    would not return, the oracle says so."""
    import numpy as np
    arrays, index = golden
    assert len(index["compose"]) > 100
    for rec in index["compose"]:
        k = rec["key"]
        R = arrays[k + "_R"]
        if rec["kind"] == "vertex":
            out, info = O.vertex_compose(R, arrays[k + "_u"], arrays[k + "_v"], rec["c"])
        else:
            out, info = O.edge_compose(R, rec["alpha"], rec["beta"], rec["rel"])
        if rec.get("hang"):
            assert info[0] == 1 and info[7] & O.EV_HANG, rec
        elif "error" in rec:
            assert info[0] != 0, rec
            if rec["error"] == "OverflowError":
                assert info[0] == 1, rec
        else:
            assert info[0] == 0, rec
            assert (out == arrays[k + "_out"]).all(), rec
        if k + "_cy" in arrays.files:
            if rec["kind"] == "vertex":
                cy = O.vertex_compose_cy(R, arrays[k + "_u"], arrays[k + "_v"], rec["c"])
            else:
                cy = O.edge_compose_cy(R, rec["alpha"], rec["beta"], rec["rel"])
            assert (cy == arrays[k + "_cy"]).all(), rec


def test_oracle_orderings_vs_golden(golden):
    """The ordering restatements (canonical sort keys, dense and sparse permutation, the
    depth-first topological sort) against the reference's outputs."""
    import numpy as np
    import scipy.sparse as sp
    arrays, index = golden
    for rec in index["ordering"]:
        k = rec["key"]
        M = arrays[k + "_A"]
        q = {int(c): v for c, v in rec["q_dense"].items()}
        # component labels: numbered by least vertex, edges both ways
        from scipy.sparse.csgraph import connected_components
        _, lab = connected_components(sp.csr_matrix(M != 0), directed=True, connection="weak")
        first = {}
        ids = np.array([first.setdefault(c, len(first)) for c in lab])
        assert {c: int((ids == c).sum()) for c in set(ids.tolist())} == q
        p = O.canonical_permutation(M, q, ids)
        assert (np.array(p) == arrays[k + "_perm_dense"]).all()
        assert (np.array(O.canonical_permutation(sp.csr_matrix(M), q, ids)) == arrays[k + "_perm_sparse"]).all()
        assert (O.permute_dense(M, p) == arrays[k + "_B_dense"]).all()
        rp = arrays[k + "_rp"]
        assert (O.permute_dense(M, rp) == arrays[k + "_permute_full"]).all()
        assert (O.permute_dense(M, rp, upper=True) == arrays[k + "_permute_upper"]).all()
        assert (O.topological_sort_dfs(sp.csr_matrix(M)) == arrays[k + "_topo"]).all()
