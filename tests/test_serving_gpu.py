"""Relationship lookups and the serving loop on the GPU: lookups against the reference's golden
answers, and every served result equal to the same request handled alone."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_golden_relationships(native, golden):
    from redblackgraph_gb300.device import to_device
    from redblackgraph_gb300.relationship import calculate_relationship, lookup_many
    arrays, index = golden
    for rec in index["relationship"]:
        W = arrays[rec["key"] + "_W"]
        Wd = to_device(W)
        got = lookup_many([(Wd, u, v) for u, v, _, _ in rec["pairs"]])
        for (u, v, ca, name), r in zip(rec["pairs"], got):
            assert (r.common_ancestor, r.relationship) == (ca, name), (rec["key"], u, v)
        for u, v, ca, name in rec["pairs"][:5]:
            r = calculate_relationship(W[u], W[v])
            assert (r.common_ancestor, r.relationship) == (ca, name)


def test_reference_relationship_examples(native):
    """Known answers of the reference's own tests (tests/reference/test_calc_relationship.py)."""
    from redblackgraph_gb300.relationship import calculate_relationship
    cases = [([-1, 0], [2, 1], 0, "parent"), ([-1, 0], [4, 1], 0, "grandparent"),
             ([1, 0], [11, -1], 0, "great grandparent"), ([1, 0], [16, -1], 0, "2nd great grandparent"),
             ([1, 0], [64, -1], 0, "4th great grandparent"),
             ([-1, 0, 2], [0, -1, 2], 2, "sibling"), ([-1, 0, 4], [0, -1, 2], 2, "aunt/uncle"),
             ([-1, 0, 8], [0, -1, 8], 2, "2nd cousin"), ([-1, 0, 4], [0, -1, 8], 2, "1st cousin 1 removed"),
             ([-1, 0], [0, -1], -1, "No Relationship")]
    for a, b, ca, name in cases:
        r = calculate_relationship(a, b)
        assert (r.common_ancestor, r.relationship) == (ca, name)


def _alone(payload, n):
    """The graph closed by itself through the single-graph entry point."""
    import scipy.sparse as sp
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    from redblackgraph_gb300.serving import storage_dtype
    ip, ij, iv = payload
    A = sp.csr_matrix((iv, ij, ip), shape=(n, n)).toarray().astype(storage_dtype(n))
    out, res = fw_dense(to_device(A))
    return A, to_host(out), int(res.status), int(res.diameter)


@pytest.mark.parametrize("inflight", [1, 2])
def test_served_results_equal_alone(native, inflight):
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Server, make_stream
    allreq = make_stream(160, 4000.0, 0.5, 32, 4600, seed=10, warm=6)
    warm, reqs = allreq[:6], allreq[6:]
    cap = 600 << 20
    ex = GpuExecutor(arena_bytes=cap, slots=inflight, keep=True)
    ex.prepare(allreq)
    srv = Server(ex, cap, Policy(inflight=inflight, max_batch=64))
    srv.run(warm)
    st = srv.run(reqs)
    assert st.batches >= 2 and st.closures + st.lookups == len(reqs)
    closed = {}
    for r in allreq:
        if r.kind != "closure":
            continue
        A, W, status, diam = _alone(ex.payloads[r.rid], r.n)
        assert r.result == (status, diam), r.rid
        assert (ex.kept[r.rid] == W).all(), r.rid
        closed[r.rid] = W
        if r.n <= 600:                             # and the alone result against the oracle
            Wo, do, so, _ = O.warshall(A)
            assert so == 0 and (Wo == W).all() and do == diam
    for r in reqs:
        if r.kind == "lookup":
            W = closed[r.target]
            assert (r.result.common_ancestor, r.result.relationship) == O.calculate_relationship(W[r.u], W[r.v])
    ex.close()


def test_unbatched_baseline_and_eviction(native):
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Server, make_stream
    reqs = make_stream(60, 3000.0, 0.4, 64, 900, seed=12)
    cap = 8 << 20                                  # small budget: graphs get evicted and reloaded
    ex = GpuExecutor(arena_bytes=cap, slots=1, keep=True)
    ex.prepare(reqs)
    st = Server(ex, cap, Policy.unbatched_baseline()).run(reqs)
    assert st.max_batch == 1 and st.evictions > 0
    for r in reqs:
        if r.kind == "closure":
            _, W, status, diam = _alone(ex.payloads[r.rid], r.n)
            assert r.result == (status, diam) and (ex.kept[r.rid] == W).all()
        else:
            W = ex.kept[r.target]
            assert (r.result.common_ancestor, r.result.relationship) == O.calculate_relationship(W[r.u], W[r.v])
    ex.close()


def test_served_mutations_match_sequential_oracle(native):
    """Links and vertex additions served among lookups: every lookup answers on the graph as
    changed by the mutations that arrived before it, and the resident closures end equal to the
    oracle's compositions applied one after another in arrival order (a link against an
    existing path is refused with the cycle status and changes nothing)."""
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Server, make_stream
    allreq = make_stream(300, 5000.0, 0.7, 24, 400, seed=21, warm=8, mutation_fraction=0.35)
    warm, reqs = allreq[:8], allreq[8:]
    cap = 256 << 20
    ex = GpuExecutor(arena_bytes=cap, slots=2, keep=True)
    ex.prepare(allreq)
    srv = Server(ex, cap, Policy(inflight=2, max_batch=32))
    srv.run(warm)
    st = srv.run(reqs)
    assert st.mutations > 20
    state = {}
    for r in sorted(allreq, key=lambda r: (r.arrival, r.rid)):
        if r.kind == "closure":
            state[r.rid] = ex.kept[r.rid].copy()       # closed alone: checked by the test above
            continue
        W = state[r.target]
        if r.kind == "lookup":
            assert (r.result.common_ancestor, r.result.relationship) == O.calculate_relationship(W[r.u], W[r.v])
        elif r.kind == "link":
            if W[r.v, r.u] != 0:
                assert r.result == _lib.RBG_ERR_CYCLE, r
                continue
            out, info = O.edge_compose(W, r.u, r.v, r.rel)
            assert r.result == int(info[0]), r
            if info[0] == 0:
                state[r.target] = out
        else:
            n = W.shape[0]
            u = np.zeros(n, W.dtype)
            u[r.u], u[r.v] = 2, 3
            out, info = O.vertex_compose(W, u, np.zeros(n, W.dtype), r.rel)
            assert r.result == int(info[0]), r
            if info[0] == 0:
                state[r.target] = out
    for gid, W in state.items():
        g = srv.store.get(gid)
        if g is not None and g.state == "closed":
            assert (ex.view(g).cpu().numpy() == W).all(), gid
    ex.close()


def test_batches_on_two_slots_overlap_on_the_gpu(native):
    """A burst of int32 closures (all on the DAG path) with two closure slots: batches of the two
    slots run on the GPU at the same time (CUDA events on each slot's stream: one batch starts
    before the other ends), and every served closure equals the request closed alone."""
    import torch
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Request, Server
    rng = np.random.default_rng(17)
    reqs = [Request(k, "closure", 0.0005 * k, n=int(rng.integers(1500, 4000)), seed=int(rng.integers(1 << 30)))
            for k in range(16)]
    cap = 4 << 30
    ex = GpuExecutor(arena_bytes=cap, slots=2, keep=True, timeline=True)
    ex.prepare(reqs)
    Server(ex, cap, Policy(inflight=2, max_batch=4)).run(reqs)
    torch.cuda.synchronize()
    tl = ex.timeline
    assert len({slot for slot, _, _ in tl}) == 2 and len(tl) >= 4
    ref = tl[0][1]
    iv = [(slot, ref.elapsed_time(a), ref.elapsed_time(b)) for slot, a, b in tl]
    overlaps = [(i, j) for i, (si, ai, bi) in enumerate(iv) for j, (sj, aj, bj) in enumerate(iv)
                if si != sj and i < j and max(ai, aj) < min(bi, bj)]
    assert overlaps, iv
    for r in reqs:
        _, W, status, diam = _alone(ex.payloads[r.rid], r.n)
        assert r.result == (status, diam) and (ex.kept[r.rid] == W).all()
    ex.close()
