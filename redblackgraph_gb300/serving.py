"""Closure and relationship-lookup serving on one GPU, with continuous batching.

Requests arrive over time (a seeded Poisson stream): a *closure* request brings a pedigree
graph (CSR) to be closed and kept resident; a *lookup* request asks the relationship of two
vertices of a graph closed earlier.  The server

* keeps closed graphs resident in one device arena (a first-fit extent allocator over a single
  HBM buffer whose size is the memory budget) and evicts the least recently used closed graph
  that no queued lookup needs when an admission does not fit;
* admits closure requests first come, first served as an in-flight slot and arena space free up,
  packing every request that has arrived (up to the batch limits) into one batched closure:
  one densify launch writes all their dense blocks straight into the arena, and one
  ``rbg_fw_batch`` call per storage type (int32 up to 4096 vertices, int64 above) closes them
  in place;
* runs up to ``inflight`` closure batches at once, each on its own CUDA stream and host worker,
  while the main loop keeps admitting; lookups on closed graphs go out in batches on a further
  stream (``rbg_relationship_lookup``), overlapping the closures on the device;
* applies *mutations* of resident closed graphs without closing them again: a *link* request
  adds the relationship u -> v (value ``rel``) to a graph (``rbg_edge_compose``, in place), an
  *add* request adds a new vertex with parents u and v and colour ``rel`` (``rbg_vertex_compose``
  into an (n+1) x (n+1) extent, the old extent released when it completes).  Mutations and
  lookups leave one queue in arrival order on one stream, so a lookup sees exactly the mutations
  that arrived before it.  A mutated graph is no longer evicted (its mutations cannot be
  regenerated from its seed);
* records each request's latency (arrival to completion) for p50/p99 reporting.

The same server with ``Policy.unbatched_baseline()`` handles one request at a time with one
closure launch per graph: the per-request baseline.

The host-side parts (arena, store, scheduler, stream generation, statistics) need no GPU; the
executor is the only part that touches the device.
"""
from __future__ import annotations

import bisect
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

ALIGN = 256


# ------------------------------------------------------------------------------ requests
@dataclass
class Request:
    rid: int
    kind: str                       # "closure", "lookup", "link" or "add"
    arrival: float                  # seconds after the start of the stream
    n: int = 0                      # closure: vertices
    seed: int = 0                   # closure: pedigree seed
    target: int = -1                # lookup / link / add: rid of the closure request of its graph
    u: int = 0                      # lookup: the two vertices; link: u -> v; add: the parents
    v: int = 0
    rel: int = 0                    # link: relationship value (2 or 3); add: colour (-1 or 1)
    done: float = math.nan          # completion, seconds after the start
    result: object = None           # closure: (status, diameter); lookup: Relationship;
                                    # link / add: status (0, or the RBG_ERR_* the change would raise)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def storage_dtype(n: int):
    """int32 up to 4096 vertices, int64 above."""
    return np.dtype(np.int32) if n <= 4096 else np.dtype(np.int64)


def make_stream(count: int, rate: float, lookup_fraction: float, lo: int, hi: int, seed: int,
                warm: int = 0, mutation_fraction: float = 0.0) -> list[Request]:
    """Seeded request stream: ``warm`` closure requests at time 0 (closed before measuring),
    then ``count`` requests with exponential inter-arrival times of mean 1/rate.  Sizes are
    log-uniform in [lo, hi]; a lookup reads two distinct vertices of a graph whose closure
    request arrived before it.  A ``mutation_fraction`` of the non-closure requests are
    mutations of such a graph, half links between two of its vertices, half new vertices with
    two of its vertices as parents."""
    rng = np.random.default_rng(seed)
    mrng = np.random.default_rng(seed + 7_777_777)   # the mutation draws leave the base stream as it is
    reqs: list[Request] = []
    closures: list[int] = []
    for k in range(warm):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        reqs.append(Request(k, "closure", 0.0, n=n, seed=int(rng.integers(2**31 - 1))))
        closures.append(k)
    t = 0.0
    for k in range(warm, warm + count):
        t += float(rng.exponential(1.0 / rate))
        if closures and rng.random() < lookup_fraction:
            g = closures[int(rng.integers(len(closures)))]
            n = reqs[g].n
            u, v = (int(x) for x in rng.choice(n, size=2, replace=False))
            if mutation_fraction > 0 and mrng.random() < mutation_fraction:
                if mrng.random() < 0.5:
                    reqs.append(Request(k, "link", t, target=g, u=u, v=v, rel=int(2 + mrng.integers(2))))
                else:
                    reqs.append(Request(k, "add", t, target=g, u=u, v=v, rel=int(-1 if mrng.random() < 0.5 else 1)))
            else:
                reqs.append(Request(k, "lookup", t, target=g, u=u, v=v))
        else:
            n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
            reqs.append(Request(k, "closure", t, n=n, seed=int(rng.integers(2**31 - 1))))
            closures.append(k)
    return reqs


def percentiles(values, qs=(50, 99)) -> dict:
    """Nearest-rank percentiles."""
    v = np.sort(np.asarray(values, dtype=np.float64))
    if v.size == 0:
        return {f"p{q}": None for q in qs}
    return {f"p{q}": float(np.percentile(v, q, method="inverted_cdf")) for q in qs}


# ------------------------------------------------------------------------------ arena
class Arena:
    """First-fit extent allocator over [0, capacity) bytes (host bookkeeping only; the bytes
    are one device buffer).  Extents are ALIGN-byte aligned; freed extents coalesce."""

    def __init__(self, capacity: int):
        self.capacity = int(capacity) // ALIGN * ALIGN
        self._free_off = [0]               # sorted offsets of free extents
        self._free_len = {0: self.capacity}
        self.used = 0

    @staticmethod
    def round(nbytes: int) -> int:
        return max(ALIGN, (int(nbytes) + ALIGN - 1) // ALIGN * ALIGN)

    def alloc(self, nbytes: int):
        need = self.round(nbytes)
        for off in self._free_off:
            ln = self._free_len[off]
            if ln >= need:
                self._free_off.remove(off)
                del self._free_len[off]
                if ln > need:
                    bisect.insort(self._free_off, off + need)
                    self._free_len[off + need] = ln - need
                self.used += need
                return off
        return None

    def release(self, off: int, nbytes: int) -> None:
        ln = self.round(nbytes)
        self.used -= ln
        i = bisect.bisect_left(self._free_off, off)
        if i < len(self._free_off) and self._free_off[i] == off + ln:     # merge with the next
            nxt = self._free_off.pop(i)
            ln += self._free_len.pop(nxt)
        if i > 0:                                                          # merge with the previous
            prev = self._free_off[i - 1]
            if prev + self._free_len[prev] == off:
                self._free_len[prev] += ln
                return
        bisect.insort(self._free_off, off)
        self._free_len[off] = ln

    def largest_free(self) -> int:
        return max(self._free_len.values(), default=0)


@dataclass
class Resident:
    gid: int
    n: int
    dtype: np.dtype
    offset: int
    nbytes: int
    state: str = "loading"          # "loading" -> "closed"
    last_use: float = 0.0
    pins: int = 0                   # queued lookups that need this graph
    status: int = 0
    diameter: int = 0
    mutated: bool = False           # changed by a link / add: never evicted


class GraphStore:
    """Resident graphs in the arena, with LRU eviction of closed, unpinned graphs."""

    def __init__(self, arena: Arena):
        self.arena = arena
        self.graphs: dict[int, Resident] = {}
        self.evictions = 0

    def get(self, gid):
        return self.graphs.get(gid)

    def reserve(self, gid: int, n: int, dtype, now: float):
        """Room for graph gid (n x n of dtype), evicting LRU closed unpinned graphs as needed;
        None when it cannot fit even then (the request waits)."""
        nbytes = n * n * np.dtype(dtype).itemsize
        if Arena.round(nbytes) > self.arena.capacity:
            raise MemoryError(f"a {n}-vertex graph does not fit in the memory budget")
        off = self.arena.alloc(nbytes)
        if off is None:
            victims = self._victims()
            for g in victims:
                self.evict(g.gid)
                off = self.arena.alloc(nbytes)
                if off is not None:
                    break
        if off is None:
            return None
        r = Resident(gid, n, np.dtype(dtype), off, nbytes, last_use=now)
        self.graphs[gid] = r
        return r

    def _victims(self, keep: int = -1):
        return sorted((g for g in self.graphs.values()
                       if g.state == "closed" and g.pins == 0 and not g.mutated and g.gid != keep),
                      key=lambda g: g.last_use)

    def grow(self, gid: int, n: int, now: float):
        """A new extent for graph gid at n x n (its dtype), evicting other LRU graphs as needed;
        returns its offset, or None when it cannot fit now.  The caller moves the graph and then
        calls ``moved``."""
        g = self.graphs[gid]
        nbytes = n * n * g.dtype.itemsize
        if Arena.round(nbytes) > self.arena.capacity:
            raise MemoryError(f"a {n}-vertex graph does not fit in the memory budget")
        off = self.arena.alloc(nbytes)
        if off is None:
            for v in self._victims(keep=gid):
                self.evict(v.gid)
                off = self.arena.alloc(nbytes)
                if off is not None:
                    break
        return off

    def moved(self, gid: int, n: int, offset: int, now: float) -> None:
        """Graph gid now lives at `offset` with n vertices; its old extent is released."""
        g = self.graphs[gid]
        self.arena.release(g.offset, g.nbytes)
        g.n, g.offset, g.nbytes, g.last_use = n, offset, n * n * g.dtype.itemsize, now

    def evict(self, gid: int) -> None:
        g = self.graphs.pop(gid)
        self.arena.release(g.offset, g.nbytes)
        self.evictions += 1


# ------------------------------------------------------------------------------ scheduling
@dataclass
class Policy:
    max_batch: int = 1024                 # graphs per closure batch
    max_batch_cells: int = 1 << 31        # sum of n^2 per batch (bounds the batch workspace)
    inflight: int = 2                     # closure batches on the device at once
    lookup_batch: int = 4096              # lookups per launch
    unbatched: bool = False               # one launch per graph (the per-request baseline)

    @classmethod
    def unbatched_baseline(cls) -> "Policy":
        return cls(max_batch=1, inflight=1, lookup_batch=1, unbatched=True)


@dataclass
class Job:
    gid: int
    n: int
    seed: int
    req: Request | None = None            # None: a reload of an evicted graph


@dataclass
class ServeStats:
    requests: int = 0
    closures: int = 0
    lookups: int = 0
    mutations: int = 0
    batches: int = 0
    lookup_launches: int = 0
    max_batch: int = 0
    evictions: int = 0
    reloads: int = 0
    peak_arena_bytes: int = 0
    makespan_s: float = 0.0
    relaxations: float = 0.0
    latency_ms: dict = field(default_factory=dict)


class Server:
    """Continuous-batching request loop over an executor (GPU or a stand-in)."""

    def __init__(self, executor, arena_bytes: int, policy: Policy | None = None):
        self.ex = executor
        self.policy = policy or Policy()
        self.store = GraphStore(Arena(arena_bytes))
        self.graph_of: dict[int, Request] = {}      # gid -> its closure request
        self.want: dict[int, int] = {}               # gid -> queued lookups needing it

    def _pin(self, gid):
        self.want[gid] = self.want.get(gid, 0) + 1
        g = self.store.get(gid)
        if g is not None:
            g.pins += 1

    def _unpin(self, gid):
        self.want[gid] -= 1
        g = self.store.get(gid)
        if g is not None:
            g.pins -= 1

    def run(self, requests: list[Request], clock=time.perf_counter) -> ServeStats:
        """Serve ``requests`` in real time (arrivals relative to the call); fills each request's
        ``done`` and ``result``.  Graphs stay resident between calls.  Returns the run's
        statistics."""
        P = self.policy
        for r in requests:
            if r.kind == "closure":
                self.graph_of[r.rid] = r
        pending = deque(sorted(requests, key=lambda r: (r.arrival, r.rid)))
        closure_q: deque[Job] = deque()
        queued: set[int] = set()                     # gids waiting in closure_q or in flight
        waiting: dict[int, list[Request]] = {}       # gid -> lookups waiting for its closure
        ready: deque[Request] = deque()
        inflight: list = []                          # (future, jobs)
        lookup_inflight = None                       # (future, lookups or [mutation], new extent)
        mutation_next = False                        # a mutation waits: it goes before more lookups
        st = ServeStats(requests=len(requests))
        remaining = len(requests)
        t0 = clock()

        def enqueue_closure(gid, req):
            g = self.graph_of[gid]
            closure_q.append(Job(gid, g.n, g.seed, req))
            queued.add(gid)

        while remaining:
            t = clock() - t0
            while pending and pending[0].arrival <= t:
                r = pending.popleft()
                if r.kind == "closure":
                    st.closures += 1
                    enqueue_closure(r.rid, r)
                    continue
                if r.kind == "lookup":
                    st.lookups += 1
                else:
                    st.mutations += 1
                self._pin(r.target)
                g = self.store.get(r.target)
                if g is not None and g.state == "closed":
                    ready.append(r)
                else:
                    waiting.setdefault(r.target, []).append(r)
                    if g is None and r.target not in queued:    # evicted: load it again
                        st.reloads += 1
                        enqueue_closure(r.target, None)
            progressed = False
            # ---- completions
            for item in [x for x in inflight if x[0].done()]:
                inflight.remove(item)
                fut, jobs = item
                results, t_done = fut.result()
                for job, (status, diameter) in zip(jobs, results):
                    g = self.store.get(job.gid)
                    g.state, g.status, g.diameter, g.last_use = "closed", status, diameter, t_done
                    queued.discard(job.gid)
                    if job.req is not None:
                        job.req.done, job.req.result = t_done, (status, diameter)
                        remaining -= 1
                    ready.extend(waiting.pop(job.gid, []))
                progressed = True
            if lookup_inflight is not None and lookup_inflight[0].done():
                fut, lks, new_off = lookup_inflight
                out, t_done = fut.result()
                if lks[0].kind == "lookup":
                    for r, rel in zip(lks, out):
                        r.done, r.result = t_done, rel
                        g = self.store.get(r.target)
                        if g is not None:
                            g.last_use = t_done
                        self._unpin(r.target)
                        remaining -= 1
                else:                                   # one mutation
                    r = lks[0]
                    g = self.store.get(r.target)
                    if r.kind == "add" and out == 0:
                        self.store.moved(r.target, g.n + 1, new_off, t_done)
                    elif r.kind == "add":
                        self.store.arena.release(new_off, (g.n + 1) * (g.n + 1) * g.dtype.itemsize)
                    g.mutated |= out == 0
                    g.last_use = t_done
                    r.done, r.result = t_done, out
                    self._unpin(r.target)
                    remaining -= 1
                lookup_inflight = None
                progressed = True
            # ---- lookups and mutations on closed graphs, one stream: a lookup never passes a
            # mutation of its own graph that arrived before it; lookups of other graphs do, and
            # a pending mutation goes out after at most one lookup batch
            if lookup_inflight is None and ready:
                mut = None
                if mutation_next:
                    # the oldest mutation with no earlier lookup of its graph still queued
                    before = set()
                    for r in ready:
                        if r.kind == "lookup":
                            before.add(r.target)
                        elif r.target not in before:
                            mut = r
                            break
                        else:
                            before.add(r.target)
                lks = []
                if mut is None:
                    blocked = set()
                    for r in ready:
                        if r.kind != "lookup":
                            blocked.add(r.target)
                        elif r.target not in blocked:
                            lks.append(r)
                            if len(lks) == P.lookup_batch:
                                break
                if lks:
                    taken = set(id(r) for r in lks)
                    ready = deque(r for r in ready if id(r) not in taken)
                    items = [(self.store.get(r.target), r.u, r.v) for r in lks]
                    lookup_inflight = (self.ex.lookups_async(items, t0), lks, None)
                    st.lookup_launches += 1
                    mutation_next = True
                    progressed = True
                else:
                    # no lookup can go: the head of the queue is a mutation
                    r = mut if mut is not None else ready[0]
                    g = self.store.get(r.target)
                    new_off = None
                    if r.kind == "add":
                        new_off = self.store.grow(r.target, g.n + 1, t)
                        st.peak_arena_bytes = max(st.peak_arena_bytes, self.store.arena.used)
                    if r.kind == "link" or new_off is not None:
                        ready.remove(r)
                        lookup_inflight = (self.ex.mutate_async(g, r, new_off, t0), [r], new_off)
                        mutation_next = False
                        progressed = True
                    elif not inflight:
                        raise MemoryError("serving stalled: a grown graph does not fit in the budget")
            # ---- closure batches
            while len(inflight) < P.inflight and closure_q:
                jobs, cells = [], 0
                while closure_q and len(jobs) < P.max_batch:
                    job = closure_q[0]
                    if jobs and cells + job.n * job.n > P.max_batch_cells:
                        break
                    g = self.store.reserve(job.gid, job.n, storage_dtype(job.n), t)
                    if g is None:
                        break                       # waits for memory (first come, first served)
                    g.pins = self.want.get(job.gid, 0)
                    closure_q.popleft()
                    jobs.append(job)
                    cells += job.n * job.n
                if not jobs:
                    break
                st.peak_arena_bytes = max(st.peak_arena_bytes, self.store.arena.used)
                st.batches += 1
                st.max_batch = max(st.max_batch, len(jobs))
                st.relaxations += float(sum(j.n ** 3 for j in jobs if j.req is not None))
                res = [self.store.get(j.gid) for j in jobs]
                inflight.append((self.ex.close_async(jobs, res, t0, P.unbatched), jobs))
                progressed = True
            if not progressed:
                if not inflight and lookup_inflight is None and not pending and closure_q and not ready:
                    raise RuntimeError("serving stalled: the queued graph does not fit in the budget")
                time.sleep(20e-6)
        st.evictions = self.store.evictions
        if requests:
            st.makespan_s = max(r.done for r in requests) - min(r.arrival for r in requests)
        st.latency_ms = {
            "all": percentiles([r.latency * 1e3 for r in requests]),
            "closure": percentiles([r.latency * 1e3 for r in requests if r.kind == "closure"]),
            "lookup": percentiles([r.latency * 1e3 for r in requests if r.kind == "lookup"]),
        }
        if st.mutations:
            st.latency_ms["mutation"] = percentiles([r.latency * 1e3 for r in requests
                                                     if r.kind in ("link", "add")])
        return st


# ------------------------------------------------------------------------------ GPU executor
class GpuExecutor:
    """Runs closure batches and lookup batches on the GPU.

    The arena is one device buffer; a resident graph is the n x n block at its extent.  Each
    closure slot owns a CUDA stream, a workspace and a host worker thread; lookups have their
    own stream and worker.  ``keep`` copies every closed graph back to the host (tests).
    ``timeline`` records, per closure batch, (slot, start, end) CUDA events on the slot's stream
    around its device work, to show when batches overlap on the GPU.
    """

    def __init__(self, arena_bytes: int, slots: int = 2, device=None, keep: bool = False,
                 timeline: bool = False):
        import threading
        from concurrent.futures import ThreadPoolExecutor
        import torch
        from . import _lib
        from .device import Workspace, require_cuda
        self.torch = torch
        self.lib = _lib
        self.L = _lib.load()
        self.device = device or require_cuda()
        self.buf = torch.empty(max(int(arena_bytes), ALIGN), dtype=torch.uint8, device=self.device)
        self.base = self.buf.data_ptr()
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.ws = [Workspace() for _ in range(slots)]
        self.free = deque(range(slots))
        self.lock = threading.Lock()
        self.pool = ThreadPoolExecutor(max_workers=slots + 1)
        self.lstream = torch.cuda.Stream(self.device)
        self.payloads: dict[int, tuple] = {}
        self.keep = keep
        self.kept: dict[int, np.ndarray] = {}
        self.timeline = [] if timeline else None

    # -- graph payloads (pedigree CSR, generated from (n, seed) and cached)
    def payload(self, gid: int, n: int, seed: int):
        p = self.payloads.get(gid)
        if p is None:
            from .synth import generations_for, pedigree_csr
            m = pedigree_csr(n, generations_for(n), seed)
            p = (np.asarray(m.indptr, dtype=np.int64), np.asarray(m.indices, dtype=np.int32),
                 np.asarray(m.data, dtype=np.int32))
            self.payloads[gid] = p
        return p

    def prepare(self, requests) -> None:
        """Generate the payloads of all closure requests ahead of time."""
        for r in requests:
            if r.kind == "closure":
                self.payload(r.rid, r.n, r.seed)

    # -- closures
    def close_async(self, jobs, residents, t0, unbatched=False):
        with self.lock:
            slot = self.free.popleft()
        return self.pool.submit(self._close, slot, jobs, residents, t0, unbatched)

    def _close(self, slot, jobs, residents, t0, unbatched):
        torch = self.torch
        try:
            with torch.cuda.stream(self.streams[slot]):
                if self.timeline is not None:
                    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                    ev[0].record(self.streams[slot])
                out = [None] * len(jobs)
                for dt in (np.dtype(np.int32), np.dtype(np.int64)):
                    idx = [k for k, g in enumerate(residents) if g.dtype == dt]
                    if idx:
                        self._close_group(slot, dt, [jobs[k] for k in idx], [residents[k] for k in idx],
                                          unbatched, out, idx)
                if self.timeline is not None:
                    ev[1].record(self.streams[slot])
                    with self.lock:
                        self.timeline.append((slot, ev[0], ev[1]))
                if self.keep:
                    for g in residents:
                        self.kept[g.gid] = self.view(g).cpu().numpy()
            return out, time.perf_counter() - t0
        finally:
            with self.lock:
                self.free.append(slot)

    def _close_group(self, slot, dt, jobs, residents, unbatched, out, idx):
        import ctypes
        L, lib = self.L, self.lib
        from .device import stream_handle, to_device
        s = self.streams[slot]
        sh = stream_handle(s)
        esz = dt.itemsize
        parts = [self.payload(j.gid, j.n, j.seed) for j in jobs]
        sizes = np.array([j.n for j in jobs], dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        nnz = np.array([p[1].size for p in parts], dtype=np.int64)
        ebase = np.concatenate([[0], np.cumsum(nnz)]).astype(np.int64)
        N = int(starts[-1])
        indptr = np.concatenate([p[0][:-1] + e for p, e in zip(parts, ebase[:-1])] + [ebase[-1:]])
        indices = np.concatenate([p[1] + st for p, st in zip(parts, starts[:-1])]).astype(np.int32)
        data = np.concatenate([p[2] for p in parts]).astype(np.int32)
        label = np.repeat(np.arange(len(jobs), dtype=np.int32), sizes)
        local = (np.arange(N, dtype=np.int64) - np.repeat(starts[:-1], sizes)).astype(np.int32)
        offs = np.array([g.offset // esz for g in residents], dtype=np.int64)
        dev = self.device
        staged = [to_device(np.ascontiguousarray(a), dev, s)
                  for a in (indptr.astype(np.int64), indices, data, label, local, starts, offs)]
        d_ip, d_ij, d_iv, d_lab, d_loc, d_st, d_off = staged
        code = lib.dtype_code(dt)
        lib.check(L.rbg_cc_densify(code, N, d_ip.data_ptr(), d_ij.data_ptr(), d_iv.data_ptr(), d_lab.data_ptr(),
                                   d_loc.data_ptr(), d_st.data_ptr(), d_off.data_ptr(), self.base,
                                   self.buf.numel() // esz, sh), "densify")
        if unbatched:
            for k, g in enumerate(residents):
                nb = ctypes.c_int64(0)
                lib.check(L.rbg_fw_dense_workspace_bytes(code, g.n, 0, ctypes.byref(nb)), "workspace")
                ws = self.ws[slot].get(nb.value, dev)
                res = lib.RbgResult()
                ptr = self.base + g.offset
                lib.check(L.rbg_fw_dense(code, g.n, ptr, g.n, ptr, g.n, 0, ws.data_ptr(), ws.numel(),
                                         ctypes.byref(res), sh), "fw_dense")
                out[idx[k]] = (int(res.status), int(res.diameter))
        else:
            nb = ctypes.c_int64(0)
            lib.check(L.rbg_fw_batch_workspace_bytes(code, len(jobs), sizes.ctypes.data, 0, ctypes.byref(nb)),
                      "workspace")
            ws = self.ws[slot].get(nb.value, dev)
            results = (lib.RbgResult * len(jobs))()
            lib.check(L.rbg_fw_batch(code, len(jobs), sizes.ctypes.data, offs.ctypes.data, self.base, self.base,
                                     0, ws.data_ptr(), ws.numel(), results, sh), "fw_batch")
            for k in range(len(jobs)):
                out[idx[k]] = (int(results[k].status), int(results[k].diameter))
        s.synchronize()          # the staging tensors are released only after the stream used them
        del staged, d_ip, d_ij, d_iv, d_lab, d_loc, d_st, d_off

    def view(self, g: Resident):
        """The resident graph as an (n, n) device tensor (a view into the arena)."""
        from .device import torch_dtype
        return self.buf[g.offset:g.offset + g.nbytes].view(torch_dtype(g.dtype)).view(g.n, g.n)

    # -- lookups
    def lookups_async(self, items, t0):
        return self.pool.submit(self._lookups, items, t0)

    def _lookups(self, items, t0):
        from .device import to_device
        from .relationship import decode, lookup_table
        torch, lib = self.torch, self.lib
        table = (lib.RbgLookup * len(items))()
        dts = []
        for k, (g, u, v) in enumerate(items):
            table[k] = lib.RbgLookup(self.base + g.offset, g.n, g.n, g.n, int(u), int(v),
                                     lib.dtype_code(g.dtype), 0)
            dts.append(g.dtype)
        with torch.cuda.stream(self.lstream):
            d = to_device(np.frombuffer(table, dtype=np.uint8).copy(), self.device, self.lstream)
            raw = lookup_table(d, len(items), self.lstream)
        return decode(raw, dts), time.perf_counter() - t0

    # -- mutations (on the lookup stream, so they keep their order with the lookups)
    def mutate_async(self, g: Resident, req: Request, new_off, t0):
        return self.pool.submit(self._mutate, g.offset, g.n, g.dtype, req, new_off, t0)

    def _mutate(self, off, n, dtype, req, new_off, t0):
        from .composition import edge_compose_device, vertex_compose_device
        from .device import torch_dtype
        torch, lib = self.torch, self.lib
        td = torch_dtype(dtype)
        R = self.buf[off:off + n * n * dtype.itemsize].view(td).view(n, n)
        with torch.cuda.stream(self.lstream):
            if req.kind == "link":
                # the reference's wrapper refuses a link against an existing path (a cycle)
                if int(R[req.v, req.u].item()) != 0:
                    return lib.RBG_ERR_CYCLE, time.perf_counter() - t0
                _, res = edge_compose_device(R, req.u, req.v, req.rel, out=R, stream=self.lstream)
            else:
                m = n + 1
                new = self.buf[new_off:new_off + m * m * dtype.itemsize].view(td).view(m, m)
                u = torch.zeros(n, dtype=td, device=self.device)
                u[req.u], u[req.v] = 2, 3           # father, mother
                v = torch.zeros(n, dtype=td, device=self.device)
                _, res = vertex_compose_device(R, u, v, req.rel, out=new, stream=self.lstream)
            self.lstream.synchronize()
        return int(res.status), time.perf_counter() - t0

    def close(self):
        self.pool.shutdown(wait=True)
