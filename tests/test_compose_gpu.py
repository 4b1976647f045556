"""Relational composition on the GPU (rbg_vertex_compose, rbg_edge_compose) against the
reference's answers (golden) and the oracle: results bit-exact, errors of the same kind."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

_ERR = {1: OverflowError, 2: ValueError}


def _expected_error(info):
    return _ERR[int(info[0])]


def test_golden_core_and_cython(native, golden):
    import redblackgraph_gb300.core as core
    import redblackgraph_gb300.sparse as sparse
    arrays, index = golden
    for rec in index["compose"]:
        k = rec["key"]
        R = arrays[k + "_R"]
        A = core.array(R)
        if rec["kind"] == "vertex":
            u, v = arrays[k + "_u"], arrays[k + "_v"]
            _, info = O.vertex_compose(R, u, v, rec["c"])
            call = lambda: core.vertex_relational_composition(u, A, v, rec["c"])  # noqa: E731
        else:
            _, info = O.edge_compose(R, rec["alpha"], rec["beta"], rec["rel"])
            call = lambda: core.edge_relational_composition(A, rec["alpha"], rec["beta"], rec["rel"])  # noqa: E731
        if "error" in rec or rec.get("hang"):
            with pytest.raises(_expected_error(info)):
                call()
        else:
            out = call()
            assert isinstance(out, core.array)
            assert out.dtype == R.dtype
            assert (np.asarray(out) == arrays[k + "_out"]).all(), rec
        if k + "_cy" in arrays.files:
            if rec["kind"] == "vertex":
                cy = sparse.vertex_relational_composition(u, R, v, rec["c"])
            else:
                cy = sparse.edge_relational_composition(R, rec["alpha"], rec["beta"], rec["rel"])
            assert (cy == arrays[k + "_cy"]).all(), rec


def _closed_pedigree(n, gens, seed, dtype):
    from redblackgraph_gb300 import synth
    W, _, st, _ = O.warshall(synth.pedigree(n, gens, seed, dtype=np.int64))
    assert st == 0
    return W.astype(dtype)


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint32, np.int16])
def test_vertex_and_edge_vs_oracle(native, dtype):
    """Closed pedigrees of 300-700 vertices: a new vertex with two parents and two children, and a
    new edge between unrelated vertices, every result equal to the oracle's."""
    from redblackgraph_gb300.composition import vertex_compose_host, edge_compose_host
    rng = np.random.default_rng(int(np.dtype(dtype).itemsize))
    for n, gens, seed in ((300, 9, 1), (700, 12, 2)):
        W = _closed_pedigree(n, gens, seed, dtype)
        f, m = rng.choice(n, size=2, replace=False)
        u = np.zeros(n, dtype)
        u[f], u[m] = 2, 3
        up = set(np.nonzero(W[f])[0]) | set(np.nonzero(W[m])[0])
        v = np.zeros(n, dtype)
        kids = [c for c in rng.permutation(n) if c not in up and not (set(np.nonzero(W[:, c])[0]) & up)][:2]
        for c in kids:
            v[c] = 2
        out, info = O.vertex_compose(W, u, v, -1)
        if info[0]:
            with pytest.raises(_expected_error(info)):
                vertex_compose_host(u, W, v, -1)
        else:
            assert (vertex_compose_host(u, W, v, -1) == out).all()
        while True:
            a, b = rng.choice(n, size=2, replace=False)
            if W[b, a] == 0 and W[a, b] == 0:
                break
        out, info = O.edge_compose(W, a, b, 3)
        if info[0]:
            with pytest.raises(_expected_error(info)):
                edge_compose_host(W, a, b, 3)
        else:
            assert (edge_compose_host(W, a, b, 3) == out).all()
        if dtype == np.int32:
            assert (vertex_compose_host(u, W, v, 1, cython=True) == O.vertex_compose_cy(W, u, v, 1)).all()
            assert (edge_compose_host(W, a, b, 2, cython=True) == O.edge_compose_cy(W, a, b, 2)).all()


def test_in_place_growth_matches(native):
    """A resident closure grown in place (the buffer holds n + 1 rows and columns) equals the
    out-of-place composition; an edge added in place likewise; only the rectangle is updated."""
    import torch
    from redblackgraph_gb300.composition import vertex_compose_device, edge_compose_device
    n = 500
    W = _closed_pedigree(n, 10, 3, np.int32)
    u = np.zeros(n, np.int32)
    u[[10, 11]] = [2, 3]
    v = np.zeros(n, np.int32)
    exp, info = O.vertex_compose(W, u, v, 1)
    assert info[0] == 0
    buf = torch.zeros((n + 8, n + 8), dtype=torch.int32, device="cuda")
    buf[:n, :n] = torch.from_numpy(W).cuda()
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    _, res = vertex_compose_device(buf, du, dv, 1, out=buf, n=n)
    assert res.status == 0
    assert res.updated == 0                      # no row reaches the new vertex
    assert (buf[:n + 1, :n + 1].cpu().numpy() == exp).all()
    assert (buf[n + 1:].cpu().numpy() == 0).all() and (buf[:, n + 1:].cpu().numpy() == 0).all()
    # an edge into the grown closure, in place
    R2 = buf[:n + 1, :n + 1].clone()
    W2 = R2.cpu().numpy()
    a = next(a for a in range(n) if W2[n, a] == 0 and W2[a, n] == 0 and np.count_nonzero(W2[:, a]) > 2)
    exp2, info2 = O.edge_compose(W2, a, n, 2)
    assert info2[0] == 0
    _, res2 = edge_compose_device(R2, a, n, 2, out=R2)
    assert res2.status == 0 and res2.updated > 0
    assert (R2.cpu().numpy() == exp2).all()


def test_errors(native):
    """A new vertex that is its own ancestor (ValueError naming the index); an overflow in a
    narrow type (OverflowError); an operand on which the reference's MSB never returns; the
    edge wrapper's cycle check."""
    import redblackgraph_gb300.core as core
    W = _closed_pedigree(60, 7, 4, np.int32)
    u = np.zeros(60, np.int32)
    u[5] = 2
    v = np.zeros(60, np.int32)
    v[5] = 3
    _, info = O.vertex_compose(W, u, v, 1)
    assert info[0] == 2
    with pytest.raises(ValueError, match=f"Idx: {info[3]}"):
        core.vertex_relational_composition(u, core.array(W), v, 1)
    # overflow: a deep chain in int8
    n = 9
    C = np.zeros((n, n), np.int64)
    np.fill_diagonal(C, [(-1 if i % 2 == 0 else 1) for i in range(n)])
    for i in range(n - 1):
        C[i + 1, i] = 2 if i % 2 == 0 else 3
    Wc, _, _, _ = O.warshall(C)
    Wc = Wc.astype(np.int8)
    uu = np.zeros(n, np.int8)
    uu[n - 1] = 2
    _, info = O.vertex_compose(Wc, uu, np.zeros(n, np.int8), 1)
    assert info[0] == 1
    with pytest.raises(OverflowError):
        core.vertex_relational_composition(uu, core.array(Wc), np.zeros(n, np.int8), 1)
    # a negative operand other than -1 (the reference would not return)
    Wn = W.copy()
    Wn[7, 3] = -5
    un = np.zeros(60, np.int32)
    un[7] = 2
    _, info = O.vertex_compose(Wn, un, np.zeros(60, np.int32), 1)
    assert info[0] == 1 and info[7] & O.EV_HANG
    with pytest.raises(OverflowError, match="does not return"):
        core.vertex_relational_composition(un, core.array(Wn), np.zeros(60, np.int32), 1)
    # the edge wrapper refuses an edge against an existing path
    a, b = [(i, j) for i in range(60) for j in range(60) if i != j and W[i, j] != 0][0]
    with pytest.raises(ValueError, match="cycle"):
        core.edge_relational_composition(core.array(W), b, a, 2)


def test_edges_of_the_domain(native):
    """An empty closure grows to one vertex; an unknown vertex index is refused; unsigned and
    narrow storage types keep the C core's wrap-around of -1."""
    import redblackgraph_gb300.core as core
    from redblackgraph_gb300.composition import vertex_compose_host, edge_compose_host
    out = vertex_compose_host(np.zeros(0, np.int32), np.zeros((0, 0), np.int32), np.zeros(0, np.int32), -1)
    assert out.shape == (1, 1) and out[0, 0] == -1
    W = _closed_pedigree(40, 5, 9, np.int32)
    with pytest.raises(Exception):
        edge_compose_host(W, 40, 1, 2)
    for dt in (np.uint8, np.uint16, np.uint32, np.uint64):
        Wt = _closed_pedigree(20, 4, 2, np.int64).astype(dt)
        u = np.zeros(20, dt)
        u[3] = 2
        exp, info = O.vertex_compose(Wt, u, np.zeros(20, dt), -1)
        if info[0] == 0:
            got = core.vertex_relational_composition(u, core.array(Wt), np.zeros(20, dt), -1)
            assert got.dtype == dt and (np.asarray(got) == exp).all()
