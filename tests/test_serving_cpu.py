"""Host logic of the serving loop (arena, store, admission, batching, lookups) with a stand-in
executor: no GPU."""
import time
from concurrent.futures import Future

import numpy as np
import pytest

from redblackgraph_gb300.serving import (ALIGN, Arena, GraphStore, Policy, Request, Server, make_stream,
                                         percentiles)


def test_arena_first_fit_and_coalescing():
    rng = np.random.default_rng(0)
    a = Arena(1 << 20)
    live = {}
    for _ in range(3000):
        if live and rng.random() < 0.45:
            off = list(live)[int(rng.integers(len(live)))]
            a.release(off, live.pop(off))
        else:
            nb = int(rng.integers(1, 40000))
            off = a.alloc(nb)
            if off is None:
                continue
            assert off % ALIGN == 0
            for o, n in live.items():           # no overlap with any live extent
                assert off + Arena.round(nb) <= o or o + Arena.round(n) <= off
            live[off] = nb
        assert a.used == sum(Arena.round(n) for n in live.values())
    for off, nb in list(live.items()):
        a.release(off, nb)
    assert a.used == 0 and a.largest_free() == a.capacity   # everything merged back


def test_store_evicts_lru_closed_unpinned():
    st = GraphStore(Arena(4 * Arena.round(100 * 100 * 4)))
    gs = [st.reserve(k, 100, np.int32, now=float(k)) for k in range(4)]
    assert all(g is not None for g in gs)
    for g in gs:
        g.state = "closed"
    gs[0].pins = 1                            # a queued lookup needs graph 0
    g = st.reserve(9, 100, np.int32, now=10.0)
    assert g is not None and st.get(0) is not None and st.get(1) is None   # graph 1 was the LRU
    gs[2].state = "loading"                    # not closed yet: not evictable
    assert st.reserve(10, 100, np.int32, now=11.0) is not None    # takes graph 3's place
    assert st.get(2) is not None and st.get(3) is None and st.get(0) is not None
    assert st.reserve(11, 100, np.int32, now=12.0) is None         # nothing left to evict
    with pytest.raises(MemoryError):
        st.reserve(11, 1000, np.int32, now=12.0)


def test_make_stream_properties():
    r1 = make_stream(500, 2000.0, 0.5, 64, 16384, seed=4, warm=8)
    r2 = make_stream(500, 2000.0, 0.5, 64, 16384, seed=4, warm=8)
    assert [(r.kind, r.arrival, r.n, r.u, r.v) for r in r1] == [(r.kind, r.arrival, r.n, r.u, r.v) for r in r2]
    arr = np.array([r.arrival for r in r1[8:]])
    assert (np.diff(arr) > 0).all()
    assert abs(np.mean(np.diff(arr)) - 1 / 2000.0) < 0.3 / 2000.0
    by = {r.rid: r for r in r1}
    for r in r1:
        if r.kind == "lookup":
            t = by[r.target]
            assert t.kind == "closure" and t.arrival <= r.arrival and r.u != r.v and max(r.u, r.v) < t.n
        else:
            assert 64 <= r.n <= 16384
    frac = np.mean([r.kind == "lookup" for r in r1[8:]])
    assert 0.4 < frac < 0.6


def test_percentiles():
    p = percentiles(np.arange(1, 101))
    assert p == {"p50": 50.0, "p99": 99.0}
    assert percentiles([]) == {"p50": None, "p99": None}


class FakeExecutor:
    """Completes closures and lookups at once; records what it was given."""

    def __init__(self):
        self.batches = []
        self.lookups = []
        self.resident_at_launch = []
        self.log = []

    @staticmethod
    def _done(value):
        f = Future()
        f.set_result(value)
        return f

    def close_async(self, jobs, residents, t0, unbatched=False):
        self.batches.append([j.gid for j in jobs])
        self.resident_at_launch.append([(g.gid, g.offset, g.nbytes) for g in residents])
        return self._done(([(0, j.n % 7) for j in jobs], time.perf_counter() - t0))

    def lookups_async(self, items, t0):
        for g, u, v in items:
            assert g is not None and g.state == "closed"
        self.lookups.append([(g.gid, u, v) for g, u, v in items])
        self.log.extend(("lookup", g.gid) for g, _, _ in items)
        return self._done(([("rel", g.gid, u, v, g.n) for g, u, v in items], time.perf_counter() - t0))

    def mutate_async(self, g, req, new_off, t0):
        assert g.state == "closed"
        if req.kind == "add":
            assert new_off is not None and new_off != g.offset
        self.log.append((req.kind, g.gid))
        return self._done((0, time.perf_counter() - t0))


def test_server_completes_everything_in_order():
    reqs = make_stream(300, 20000.0, 0.5, 16, 300, seed=1)
    ex = FakeExecutor()
    st = Server(ex, 1 << 30).run(reqs)
    assert all(np.isfinite(r.done) and r.done >= r.arrival for r in reqs)
    by = {r.rid: r for r in reqs}
    for r in reqs:
        if r.kind == "lookup":
            assert r.result[:4] == ("rel", r.target, r.u, r.v)
            assert r.done >= by[r.target].done
        else:
            assert r.result == (0, r.n % 7)
    order = [g for b in ex.batches for g in b]
    closures = [r.rid for r in sorted(reqs, key=lambda r: r.arrival) if r.kind == "closure"]
    assert order == closures                        # first come, first served
    assert st.closures + st.lookups == st.requests == 300
    assert st.latency_ms["all"]["p50"] is not None


def test_server_batches_what_has_arrived():
    # a burst: everything arrives at once, so the batches are as large as the limit allows
    reqs = [Request(k, "closure", 1e-6, n=10 + k, seed=k) for k in range(50)]
    ex = FakeExecutor()
    Server(ex, 1 << 30, Policy(max_batch=20)).run(reqs)
    assert [len(b) for b in ex.batches] == [20, 20, 10]
    ex2 = FakeExecutor()
    Server(ex2, 1 << 30, Policy.unbatched_baseline()).run(
        [Request(k, "closure", 1e-6, n=10 + k, seed=k) for k in range(5)])
    assert [len(b) for b in ex2.batches] == [1] * 5


def test_server_budget_eviction_and_reload():
    # room for a few 100x100 int32 graphs: old ones are evicted, and a lookup on an evicted
    # graph reloads it before answering
    cap = 3 * 100 * 100 * 4 + ALIGN
    reqs = [Request(k, "closure", 1e-4 * (k + 1), n=100, seed=k) for k in range(6)]
    reqs.append(Request(6, "lookup", 1e-2, target=0, u=1, v=2))
    ex = FakeExecutor()
    srv = Server(ex, cap)
    st = srv.run(reqs)
    assert st.evictions >= 3 and st.reloads == 1
    assert reqs[-1].result[:4] == ("rel", 0, 1, 2)
    for snap in ex.resident_at_launch:            # extents stay inside the arena
        for gid, off, nb in snap:
            assert off + nb <= cap
    assert srv.store.arena.used <= srv.store.arena.capacity


def test_server_mutations_in_order_and_growth():
    """Links and vertex additions leave the lookup queue in arrival order (a lookup after an
    add sees the grown graph), an add moves the graph to a larger extent and frees the old one,
    and mutated graphs are not evicted."""
    reqs = make_stream(400, 20000.0, 0.6, 16, 200, seed=3, warm=5, mutation_fraction=0.3)
    kinds = {r.kind for r in reqs}
    assert {"link", "add", "lookup", "closure"} <= kinds
    ex = FakeExecutor()
    srv = Server(ex, 1 << 30)
    srv.run(reqs[:5])
    st = srv.run(reqs[5:])
    assert st.mutations == sum(r.kind in ("link", "add") for r in reqs[5:])
    assert all(np.isfinite(r.done) for r in reqs)
    # per graph, mutations and lookups were issued in arrival order
    issued = [e for e in ex.log]
    for gid in {r.target for r in reqs if r.kind != "closure"}:
        want = [(r.kind, gid) for r in sorted(reqs, key=lambda r: (r.arrival, r.rid))
                if r.kind != "closure" and r.target == gid]
        assert [e for e in issued if e[1] == gid] == want
    # a lookup answers on the graph as grown by the adds that arrived before it
    grown = {}
    for r in sorted(reqs, key=lambda r: (r.arrival, r.rid)):
        if r.kind == "closure":
            grown[r.rid] = r.n
        elif r.kind == "add":
            grown[r.target] += 1
        elif r.kind == "lookup":
            assert r.result[4] == grown[r.target], r
    for gid, n in grown.items():
        g = srv.store.get(gid)
        if g is not None:
            assert g.n == n and g.nbytes == n * n * g.dtype.itemsize
    assert srv.store.arena.used <= srv.store.arena.capacity
    mutated = [g for g in srv.store.graphs.values() if g.mutated]
    assert mutated and all(g.gid in srv.store.graphs for g in mutated)
