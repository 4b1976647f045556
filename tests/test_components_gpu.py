"""Component-wise closure on the GPU (component split, batched closure, merge) against the
reference's golden answers and the oracle, bit-exact."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(a, b):
    a, b = sp.csr_matrix(a), sp.csr_matrix(b)
    a.sort_indices()
    b.sort_indices()
    return (a.shape == b.shape and a.nnz == b.nnz and (a.indptr == b.indptr).all()
            and (a.indices == b.indices).all() and (a.data == b.data).all())


def _shuffled_forest(sizes, seed, dtype=np.int32, shuffle=True):
    from redblackgraph_gb300 import synth
    blocks = [synth.pedigree_csr(int(n), synth.generations_for(int(n)), seed + j, dtype=dtype)
              for j, n in enumerate(sizes)]
    M = sp.block_diag(blocks, format="csr")
    if not shuffle:                 # every component numbered oldest first (the DAG path)
        M.sort_indices()
        return M
    perm = np.random.default_rng(seed).permutation(M.shape[0])
    M = sp.csr_matrix(M[perm][:, perm])
    M.sort_indices()
    return M


def test_golden_component_wise_closure(native, golden):
    from redblackgraph_gb300.sparse import component_wise_closure, CycleError
    arrays, index = golden
    for rec in index["components"]:
        k, n = rec["key"], rec["n"]
        A = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]), shape=(n, n))
        if "error" in rec:
            with pytest.raises(CycleError) as ei:
                component_wise_closure(A, rec["method"], rec["threshold"])
            assert ei.value.vertex == rec["vertex"]
            continue
        r = component_wise_closure(A, method=rec["method"], densify_threshold=rec["threshold"])
        E = sp.csr_matrix((arrays[k + "_W_data"], arrays[k + "_W_indices"], arrays[k + "_W_indptr"]),
                          shape=(n, n))
        assert _same(r.W, E), rec
        assert r.W.dtype == np.int32 and r.W.has_sorted_indices
        assert r.diameter == rec["diameter"], rec


def test_labels_match_oracle(native):
    import torch
    from redblackgraph_gb300.components import label_components
    from redblackgraph_gb300.device import to_device, to_host
    M = _shuffled_forest([50, 1, 3, 400, 17, 2, 90, 1], seed=41)
    n = M.shape[0]
    c = label_components(to_device(M.indptr.astype(np.int64)), to_device(M.indices.astype(np.int32)), n)
    lab = O.components(M.indptr, M.indices, n)
    assert c.count == int(lab.max()) + 1
    assert (to_host(c.label)[:n] == lab).all()
    sv = to_host(c.sorted_vertex)[:n]
    assert (sv == np.argsort(lab, kind="stable")).all()
    st = to_host(c.start)[:c.count + 1]
    assert (np.diff(st) == np.bincount(lab)).all()
    loc = to_host(c.local)[:n]
    assert (loc[sv] == np.arange(n) - st[lab[sv]]).all()
    torch.cuda.synchronize()


@pytest.mark.parametrize("method,threshold,shuffle", [("auto", 500, True), ("auto", 100, True), ("FW", 500, True),
                                                      ("D", 500, True), ("auto", 500, False), ("FW", 500, False)])
def test_forest_vs_oracle(native, method, threshold, shuffle):
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import component_wise_closure
    sizes = synth.component_sizes(40, 4, 700, seed=5)
    M = _shuffled_forest(sizes, seed=7, shuffle=shuffle)
    r = component_wise_closure(M, method=method, densify_threshold=threshold)
    W, d, err = O.component_wise_closure(M, method, threshold)
    assert err is None
    assert _same(r.W, W)
    assert r.diameter == d


def test_single_component_and_edge_cases(native):
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sparse import component_wise_closure
    M = synth.pedigree_csr(300, 12, 9)
    for method in ("auto", "FW", "D"):
        r = component_wise_closure(M, method=method)
        W, d, err = O.component_wise_closure(M, method, 500)
        assert err is None and _same(r.W, W) and r.diameter == d
    r = component_wise_closure(sp.csr_matrix((0, 0), dtype=np.int32))
    assert r.W.shape == (0, 0) and r.diameter == 0
    E = sp.csr_matrix((5, 5), dtype=np.int32)                  # no stored entries at all
    r = component_wise_closure(E)
    assert r.W.nnz == 0 and r.diameter == 0
    # duplicate entries are summed (scipy's toarray in the reference), dense input accepted
    D = sp.coo_matrix((np.array([1, -1, 1, 1, 1]), (np.array([0, 1, 0, 2, 2]), np.array([0, 1, 1, 2, 0]))),
                      shape=(3, 3))
    r = component_wise_closure(D)
    W, d, err = O.component_wise_closure(D, "auto", 500)
    assert _same(r.W, W) and r.diameter == d
    r2 = component_wise_closure(D.toarray())
    assert _same(r2.W, W)


def test_cycle_in_a_later_component_raises(native):
    from redblackgraph_gb300.sparse import component_wise_closure, CycleError
    M = _shuffled_forest([30, 60, 25], seed=13).tolil()
    lab = O.components(sp.csr_matrix(M).indptr, sp.csr_matrix(M).indices, M.shape[0])
    verts = np.flatnonzero(lab == 1)
    sub = sp.csr_matrix(M)[verts][:, verts].tocoo()
    off = np.flatnonzero(sub.row != sub.col)[0]
    M[verts[sub.col[off]], verts[sub.row[off]]] = 2            # close a two-vertex cycle
    M = sp.csr_matrix(M)
    _, _, err = O.component_wise_closure(M)
    assert err is not None and err[0] == 1
    with pytest.raises(CycleError) as ei:
        component_wise_closure(M)
    assert ei.value.vertex == int(err[1][2])


def test_golden_adaptive_and_component_labels(native, golden):
    """transitive_closure_adaptive (components / DAG / Floyd-Warshall dispatch, the sparse_only
    error) and find_components_sparse against the reference."""
    from redblackgraph_gb300.sparse import (transitive_closure_adaptive, find_components_sparse,
                                            DensificationError)
    arrays, index = golden
    for rec in index["adaptive"]:
        k, n = rec["key"], rec["n"]
        A = sp.csr_matrix((arrays[k + "_data"], arrays[k + "_indices"], arrays[k + "_indptr"]), shape=(n, n))
        q = {}
        lab = find_components_sparse(A, q)
        assert (lab.astype(np.int64) == arrays[k + "_labels"]).all(), rec["name"]
        assert {str(c): v for c, v in q.items()} == rec["q"]
        if "error" in rec:
            with pytest.raises(DensificationError):
                transitive_closure_adaptive(A, **rec["kwargs"])
            continue
        r = transitive_closure_adaptive(A, **rec["kwargs"])
        E = sp.csr_matrix((arrays[k + "_W_data"], arrays[k + "_W_indices"], arrays[k + "_W_indptr"]), shape=(n, n))
        assert _same(r.W, E), rec["name"]
        assert r.diameter == rec["diameter"], rec["name"]


@pytest.mark.parametrize("shuffle,blocked", [(True, True), (True, False), (False, False)])
def test_recorded_row_statistics_equal_the_counting_pass(native, shuffle, blocked):
    """rbg_fw_batch_rows records, while it writes the result (finalisation of the blocked
    kernels with RBG_MODE_NO_DAG, else the DAG path's writes: components numbered oldest first,
    or shuffled and replayed in their own numbering), the row counts, chunk masks and component
    maxima that rbg_cc_compact_count would read back from the closed blocks."""
    import ctypes
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.components import label_components, densify, compact, chunk_mask_buffer
    from redblackgraph_gb300.dense import fw_batch
    from redblackgraph_gb300.device import to_device
    sizes = synth.component_sizes(30, 4, 2300, seed=11)      # rows past 2048 columns: two mask words
    M = _shuffled_forest(sizes, seed=13, shuffle=shuffle)
    n = M.shape[0]
    ip, ix, dv = (to_device(M.indptr.astype(np.int64)), to_device(M.indices.astype(np.int32)),
                  to_device(M.data.astype(np.int32)))
    comps = label_components(ip, ix, n)
    blocks = densify(ip, ix, dv, comps)
    ref = blocks.flat.clone()
    row_count = torch.full((n,), -7, dtype=torch.int64, device="cuda")
    mask = chunk_mask_buffer(comps, blocks)
    cmax = torch.zeros(comps.count, dtype=torch.int32, device="cuda")
    stats = _lib.RbgRowStats(comps.start.data_ptr(), comps.sorted_vertex.data_ptr(), row_count.data_ptr(),
                             mask.data_ptr(), cmax.data_ptr())
    mode = _lib.MODE_CYTHON | _lib.MODE_GRAPH | (_lib.MODE_NO_DAG if blocked else 0)
    _, res = fw_batch(blocks.flat, blocks.sizes, blocks.offsets, out=blocks.flat, mode=mode, as_array=True,
                      row_stats=stats)
    assert (res["status"] == 0).all()
    assert (res["path"] == (_lib.PATH_BLOCKED32 if blocked else _lib.PATH_DAG)).all()
    _, res2 = fw_batch(ref, blocks.sizes, blocks.offsets, out=ref, mode=mode, as_array=True)
    assert torch.equal(ref, blocks.flat)
    # the counting pass over the same closed blocks
    oi, oj, ov, cm = compact(comps, blocks, want_max=True)
    cnt = np.diff(oi.cpu().numpy())
    assert (row_count.cpu().numpy() == cnt).all()
    assert (cmax.cpu().numpy() == cm[:comps.count].cpu().numpy()).all()
    # the merged matrix from the recorded statistics is the same matrix
    oi2, oj2, ov2, _ = compact(comps, blocks, counted=(row_count, mask, cmax))
    assert torch.equal(oi, oi2) and torch.equal(oj, oj2) and torch.equal(ov, ov2)
    # the recorded rows after a second call are replayed from the CUDA graph: same counts
    row_count.fill_(-7)
    fw_batch(ref, blocks.sizes, blocks.offsets, out=ref, mode=mode, as_array=True, row_stats=stats)
    assert (row_count.cpu().numpy() == cnt).all()
    # the call refuses what it cannot record
    bad = _lib.RbgRowStats(comps.start.data_ptr(), None, None, None, None)
    with pytest.raises(Exception):
        fw_batch(ref, blocks.sizes, blocks.offsets, out=ref, mode=mode, row_stats=bad)
    del ctypes


def test_component_on_another_path_is_counted_again(native):
    """A component whose products leave the 32-bit lanes is closed on the exact path and has no
    recorded statistics: the merge counts every row again and the result equals the oracle's."""
    from redblackgraph_gb300.sparse import component_wise_closure
    sizes = [60, 5, 200]
    M = _shuffled_forest(sizes, seed=17).tolil()
    # a chain of three vertices whose values overflow 32 bits when composed (Cython semantics wrap)
    n0 = M.shape[0]
    M.resize((n0 + 3, n0 + 3))
    M[n0, n0] = -1
    M[n0 + 1, n0 + 1] = 1
    M[n0 + 2, n0 + 2] = -1
    M[n0, n0 + 1] = 1 << 20
    M[n0 + 1, n0 + 2] = 1 << 20
    M = sp.csr_matrix(M, dtype=np.int32)
    M.sort_indices()
    r = component_wise_closure(M)
    W, d, err = O.component_wise_closure(M)
    assert err is None
    assert _same(r.W, W)
    assert r.diameter == d


@pytest.mark.parametrize("reverse", [False, True])
def test_csr_dag_path_vs_oracle(native, reverse):
    """Components numbered in a topological order (oldest first, or reversed: entries above the
    diagonal) are closed straight from the CSR graph; results and diameters of every method
    equal the oracle's.  One component in another order sends the graph to the dense path."""
    import torch
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.components import label_components, dag_component_closure
    from redblackgraph_gb300.device import to_device
    from redblackgraph_gb300.sparse import component_wise_closure
    sizes = synth.component_sizes(50, 1, 900, seed=21)
    M = _shuffled_forest(sizes, seed=23, shuffle=False)
    n = M.shape[0]
    if reverse:
        p = np.arange(n)[::-1]
        M = sp.csr_matrix(M[p][:, p])
        M.sort_indices()
    dev = lambda a, t: to_device(np.ascontiguousarray(a).astype(t))  # noqa: E731
    ip, ix, dv = dev(M.indptr, np.int64), dev(M.indices, np.int32), dev(M.data, np.int32)
    comps = label_components(ip, ix, n)
    assert dag_component_closure(ip, ix, dv, n, comps, "auto", 500) is not None
    for method, thr in (("auto", 500), ("auto", 60), ("FW", 500), ("D", 500)):
        r = component_wise_closure(M, method=method, densify_threshold=thr)
        W, d, err = O.component_wise_closure(M, method, thr)
        assert err is None and _same(r.W, W) and r.diameter == d, (method, thr)
        assert r.W.has_sorted_indices
    # one component renumbered at random: the whole graph takes the dense path, same answers
    big = int(np.argmax(sizes))
    lo = int(np.sum(sizes[:big])) if not reverse else n - int(np.sum(sizes[:big + 1]))
    q = np.arange(n)
    q[lo:lo + int(sizes[big])] = lo + np.random.default_rng(3).permutation(int(sizes[big]))
    S = sp.csr_matrix(M[q][:, q])
    S.sort_indices()
    sip, six, sdv = dev(S.indptr, np.int64), dev(S.indices, np.int32), dev(S.data, np.int32)
    assert dag_component_closure(sip, six, sdv, n, label_components(sip, six, n), "auto", 500) is None
    r = component_wise_closure(S)
    W, d, err = O.component_wise_closure(S)
    assert err is None and _same(r.W, W) and r.diameter == d
    torch.cuda.synchronize()
