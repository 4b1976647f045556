"""Canonical ordering, permutations, topological sort and the triangularity check on the GPU,
against the reference's answers (golden) and the oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_golden_canonical_ordering_and_permute(native, golden):
    import redblackgraph_gb300.core as core
    from redblackgraph_gb300.sparse import csgraph
    from redblackgraph_gb300.types import Ordering
    arrays, index = golden
    for rec in index["ordering"]:
        k = rec["key"]
        M = arrays[k + "_A"]
        d = csgraph.avos_canonical_ordering(core.array(M))
        assert isinstance(d, Ordering)
        assert (np.asarray(d.label_permutation) == arrays[k + "_perm_dense"]).all(), k
        assert (np.asarray(d.A) == arrays[k + "_B_dense"]).all(), k
        assert {str(c): v for c, v in d.components.items()} == rec["q_dense"]
        s = csgraph.avos_canonical_ordering(sp.csr_matrix(M))
        assert (np.asarray(s.label_permutation) == arrays[k + "_perm_sparse"]).all(), k
        B = sp.csr_matrix((arrays[k + "_B_data"], arrays[k + "_B_indices"], arrays[k + "_B_indptr"]), shape=M.shape)
        assert (s.A != B).nnz == 0 and s.A.has_sorted_indices
        assert {str(c): v for c, v in s.components.items()} == rec["q_sparse"]
        rp = arrays[k + "_rp"]
        assert (csgraph.permute(M, rp) == arrays[k + "_permute_full"]).all()
        assert (csgraph.permute(M, rp, assume_upper_triangular=True) == arrays[k + "_permute_upper"]).all()
        P = sp.csr_matrix((arrays[k + "_ps_data"], arrays[k + "_ps_indices"], arrays[k + "_ps_indptr"]),
                          shape=M.shape)
        got = csgraph.permute_sparse(sp.csr_matrix(M), rp, assume_upper_triangular=True)
        assert (got != P).nnz == 0 and got.nnz == P.nnz
        # the full sparse permutation equals the dense one
        assert (csgraph.permute_sparse(sp.csr_matrix(M), rp).toarray() == arrays[k + "_permute_full"]).all()


def test_canonical_ordering_vs_oracle_at_size(native):
    """A 2,000-vertex closed forest with many equal-size components: the canonical permutation
    equals the oracle's sort."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import csgraph, transitive_closure_dag_sparse
    A = synth.forest(2000, 8, 3, family=40, reach=2, dtype=np.int32)
    W = sp.csr_matrix(transitive_closure_dag_sparse(A).W)
    q = {}
    ids = csgraph.find_components(W, q)
    exp = O.canonical_permutation(W, q, ids)
    got = csgraph._get_permutation_sparse(W, q, ids)
    assert got == exp
    o = csgraph.avos_canonical_ordering(W)
    assert list(o.label_permutation) == exp
    assert csgraph.is_upper_triangular(o.A)


def test_topological_sort_properties(native):
    """A valid permutation after which every edge lies above the diagonal; CycleError on cycles;
    topological_ordering returns the triangular matrix; is_upper_triangular on its cases."""
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import csgraph
    from redblackgraph_gb300.sparse.csgraph import CycleError
    for seed in (1, 2):
        A = synth.forest(3000, 10, seed, family=100, reach=3, dtype=np.int32)
        p = np.random.default_rng(seed).permutation(3000)
        A = sp.csr_matrix(A[p][:, p])
        t = csgraph.topological_sort(A)
        assert sorted(t.tolist()) == list(range(3000))
        B = csgraph.permute_sparse(A, t, assume_upper_triangular=True)
        assert B.nnz == A.nnz and csgraph.is_upper_triangular(B)
        o = csgraph.topological_ordering(A)
        assert csgraph.is_upper_triangular(o.A) and o.A.nnz == A.nnz
        assert isinstance(o.components, dict) and len(o.components) > 1
    assert list(csgraph.topological_sort(sp.csr_matrix(np.eye(5, dtype=np.int32)))) == [0, 1, 2, 3, 4]
    assert len(csgraph.topological_sort(sp.csr_matrix((0, 0), dtype=np.int32))) == 0
    for M in (np.array([[1, 2, 0], [0, 1, 4], [8, 0, 1]]), np.array([[1, 2], [4, 1]])):
        with pytest.raises(CycleError):
            csgraph.topological_sort(sp.csr_matrix(M.astype(np.int32)))
    U = np.array([[1, 2, 4], [0, 1, 2], [0, 0, 1]], np.int32)
    assert csgraph.is_upper_triangular(U) and not csgraph.is_upper_triangular(U.T)
    assert not csgraph.is_upper_triangular(U, strict=True)
    assert csgraph.is_upper_triangular(np.triu(U, 1), strict=True)


def test_golden_extract_and_merge(native, golden):
    """extract_submatrix of every component and merge_component_matrices back, against the
    reference's outputs."""
    from redblackgraph_gb300.sparse import csgraph
    arrays, index = golden
    for rec in index["ordering"]:
        k = rec["key"]
        S = sp.csr_matrix(arrays[k + "_A"])
        lab = csgraph.find_components_sparse(S)
        parts = []
        for c, verts in sorted(csgraph.get_component_vertices(lab).items()):
            sub, mp = csgraph.extract_submatrix(S, verts)
            exp = sp.csr_matrix((arrays[f"{k}_sub{c}_data"], arrays[f"{k}_sub{c}_indices"],
                                 arrays[f"{k}_sub{c}_indptr"]), shape=sub.shape)
            assert (sub != exp).nnz == 0 and sub.nnz == exp.nnz and sub.dtype == np.int32
            assert (mp == arrays[f"{k}_sub{c}_map"]).all()
            parts.append((sub, mp))
        assert len(parts) == rec["ncomp"]
        merged = csgraph.merge_component_matrices(parts, S.shape[0])
        exp = sp.csr_matrix((arrays[k + "_merged_data"], arrays[k + "_merged_indices"], arrays[k + "_merged_indptr"]),
                            shape=S.shape)
        assert (merged != exp).nnz == 0 and merged.nnz == exp.nnz
        assert (merged != S).nnz == 0


def test_orderings_on_tiny_graphs(native):
    """Empty and one-vertex graphs, a graph of isolated vertices (every component of size 1)."""
    from redblackgraph_gb300.sparse import csgraph
    e = sp.csr_matrix((0, 0), dtype=np.int32)
    assert len(csgraph.topological_sort(e)) == 0 and csgraph.is_upper_triangular(e)
    one = sp.csr_matrix(np.array([[-1]], np.int32))
    o = csgraph.avos_canonical_ordering(one)
    assert list(o.label_permutation) == [0] and o.components == {0: 1}
    iso = np.diag(np.array([1, -1, 1, -1, -1], np.int32))
    o = csgraph.avos_canonical_ordering(sp.csr_matrix(iso))
    q = {c: 1 for c in range(5)}
    assert list(o.label_permutation) == O.canonical_permutation(iso, q, np.arange(5))
    d = csgraph.avos_canonical_ordering(iso)
    assert list(d.label_permutation) == list(o.label_permutation)
