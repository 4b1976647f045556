"""Batched dense closure (many components in one run) against the oracle, bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run_batch(mats, mode=0, in_place=False):
    import torch
    from redblackgraph_gb300.dense import fw_batch, pack
    from redblackgraph_gb300.device import to_device, to_host
    flat, sizes, offsets = pack(mats)
    d = to_device(flat)
    out, res = fw_batch(d, sizes, offsets, out=d if in_place else None, mode=mode)
    torch.cuda.synchronize()
    h = to_host(out)
    return [h[o:o + n * n].reshape(n, n) for o, n in zip(offsets, sizes)], res


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_mixed_sizes_vs_oracle(native, dtype):
    from redblackgraph_gb300 import synth
    sizes, seeds = synth.batch_components(60, 3, 700, seed=5)
    mats = [synth.pedigree(int(n), synth.generations_for(int(n)), int(s), dtype=dtype)
            for n, s in zip(sizes, seeds)]
    Ws, res = run_batch(mats)
    for A, W, r in zip(mats, Ws, res):
        Wo, do, so, _ = O.warshall(A)
        assert r.status == so == 0
        assert (W == Wo).all() and r.diameter == do


def test_batch_with_fallbacks_in_place(native):
    """Clean, unclean (exact path), cyclic and 64-bit-wide components in one batch."""
    from redblackgraph_gb300 import synth, _lib
    mats = [synth.pedigree(n, 8, n, dtype=np.int64) for n in (10, 70, 130, 257, 1)]
    rs = np.random.RandomState(3)
    U = np.triu(rs.randint(0, 4, size=(40, 40)), k=1)
    np.fill_diagonal(U, rs.choice([-1, 1], size=40))
    mats.append(U.astype(np.int64))
    C = synth.pedigree(90, 8, 4, dtype=np.int64)
    Wc, _, _, _ = O.warshall(C)
    v, u = max(zip(*np.nonzero(np.tril(Wc, -1))), key=lambda t: t[0] - t[1])
    C[u, v] = 2
    mats.append(C)
    Wd = synth.pedigree(150, 9, 6, dtype=np.int64)
    mats.append(np.where(Wd > 1, Wd << 8, Wd))
    Ws, res = run_batch(mats, in_place=True)
    for A, W, r in zip(mats, Ws, res):
        Wo, do, so, _ = O.warshall(A)
        assert r.status == so
        if so == 0:
            assert (W == Wo).all() and r.diameter == do
    assert res[5].path == _lib.PATH_EXACT and res[6].status == _lib.RBG_ERR_CYCLE
    assert res[7].path == _lib.PATH_BLOCKED64


def test_cython_batch(native):
    from redblackgraph_gb300 import synth, _lib
    mats = [synth.pedigree(n, 7, n + 1, dtype=np.int32) for n in (33, 64, 65, 200)]
    Ws, res = run_batch(mats, mode=_lib.MODE_CYTHON)
    for A, W, r in zip(mats, Ws, res):
        Wo, do, so, _ = O.fw_cython(A)
        assert r.status == so == 0 and (W == Wo).all() and r.diameter == do


@pytest.mark.parametrize("extra", ["dag", "blocked"])
def test_graph_replay_matches_direct_launches(native, extra):
    """RBG_MODE_GRAPH: the first call records the batch's launch sequence (the DAG path with its
    level loop as a device-driven while node, or with RBG_MODE_NO_DAG the blocked kernels), later
    calls with the same sizes, offsets and buffers replay it; results (values, diameters,
    fallbacks) equal the direct launches, also after the input changes in place between
    replays."""
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_batch, pack
    from redblackgraph_gb300.device import to_device, to_host
    sizes, seeds = synth.batch_components(40, 3, 500, seed=9)
    mats = [synth.pedigree(int(n), synth.generations_for(int(n)), int(s), dtype=np.int32)
            for n, s in zip(sizes, seeds)]
    cyc = np.array([[0, 2, 0], [0, 0, 3], [2, 0, 0]], dtype=np.int32)   # a cycle: reruns alone
    mats.append(cyc)
    flat, sz, off = pack(mats)
    d = to_device(flat)
    out = torch.empty_like(d)
    base = _lib.MODE_NO_DAG if extra == "blocked" else 0
    ref, rres = fw_batch(d, sz, off, out=torch.empty_like(d), mode=base)
    ref = to_host(ref)
    L = native
    for rep in range(3):
        l0 = L.rbg_launch_count()
        _, res = fw_batch(d, sz, off, out=out, mode=_lib.MODE_GRAPH | base)
        torch.cuda.synchronize()
        assert L.rbg_launch_count() > l0                     # replays count their launches
        assert (to_host(out) == ref).all()
        assert [(r.status, r.diameter) for r in res] == [(r.status, r.diameter) for r in rres]
    # new contents, same layout: the replay reads the new input
    mats2 = [synth.pedigree(int(n), synth.generations_for(int(n)), int(s) + 1, dtype=np.int32)
             for n, s in zip(sizes, seeds)] + [cyc]
    flat2, _, _ = pack(mats2)
    d.copy_(to_device(flat2))
    _, res2 = fw_batch(d, sz, off, out=out, mode=_lib.MODE_GRAPH | base)
    torch.cuda.synchronize()
    h = to_host(out)
    for A, o, n, r in zip(mats2[:-1], off, sz, res2):
        Wo, do, so, _ = O.warshall(A)
        assert (h[o:o + n * n].reshape(n, n) == Wo).all() and r.diameter == do


@pytest.mark.parametrize("mode_name", ["MODE_TILE_NARROW", "MODE_AUTOTUNE"])
def test_tile_shapes_and_autotune_match_oracle(native, mode_name):
    """The narrow phase-3 tile shape, and the autotuned per-round shapes (the first call tunes by
    closing the batch with both shapes), give the oracle's results; a second call reuses the
    tuned shapes."""
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_batch, pack
    from redblackgraph_gb300.device import to_device, to_host
    sizes, seeds = synth.batch_components(30, 3, 900, seed=11)
    mats = [synth.pedigree(int(n), synth.generations_for(int(n)), int(s), dtype=np.int32)
            for n, s in zip(sizes, seeds)]
    flat, sz, off = pack(mats)
    d = to_device(flat)
    mode = getattr(_lib, mode_name) | _lib.MODE_NO_DAG   # the blocked kernels are the subject
    for _ in range(2):
        out, res = fw_batch(d, sz, off, out=torch.empty_like(d), mode=mode)
        torch.cuda.synchronize()
        h = to_host(out)
        for A, o, n, r in zip(mats, off, sz, res):
            Wo, do, so, _ = O.warshall(A)
            assert r.status == so == 0
            assert (h[o:o + n * n].reshape(n, n) == Wo).all() and r.diameter == do


def _random_dag(rng, n, density, above=False, vmax=8):
    """Random DAG numbered in a topological order: entries below the diagonal (or, reversed,
    above it) with values in [2, vmax), diagonal in {-1, 0, 1}."""
    A = np.zeros((n, n), np.int64)
    low = np.tril(rng.random((n, n)) < density, -1)
    A[low] = rng.integers(2, vmax, size=int(low.sum()))
    np.fill_diagonal(A, rng.choice([-1, 0, 1], size=n))
    return A[::-1, ::-1].copy() if above else A


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
@pytest.mark.parametrize("in_place", [False, True])
def test_dag_path_vs_oracle(native, in_place, dtype):
    """int32 and int64 matrices numbered in a topological order (entries all below, or all
    above, the diagonal) take the DAG path; values, diameters (each cell's first value) and
    errors equal the oracle's sequential loop, in both semantics (Cython: int32 only)."""
    from redblackgraph_gb300 import synth, _lib
    rng = np.random.default_rng(7)
    mats = [_random_dag(rng, int(rng.integers(1, 90)), rng.uniform(0.02, 0.4), above=t % 2 == 1).astype(dtype)
            for t in range(60)]
    mats += [synth.pedigree(n, synth.generations_for(n), n, dtype=dtype) for n in (300, 700, 1500)]
    mats += [synth.pedigree(500, 12, 9, dtype=dtype)[::-1, ::-1].copy()]   # pedigree above the diagonal
    semantics = ((0, O.warshall), (_lib.MODE_CYTHON, O.fw_cython)) if dtype == np.int32 else ((0, O.warshall),)
    for mode, oracle in semantics:
        Ws, res = run_batch(mats, mode=mode, in_place=in_place)
        dag = 0
        for A, W, r in zip(mats, Ws, res):
            Wo, do, so, _ = oracle(A)
            assert r.status == so
            if so == 0:
                assert (W == Wo).all() and r.diameter == do
            dag += r.path == _lib.PATH_DAG
        assert dag >= 40                     # deep random DAGs may reach the top bit: blocked path


def test_dag_path_mixed_batch_and_opt_out(native):
    """A batch mixing DAG-path matrices (numbered oldest first, youngest first, or shuffled) with
    ones that must take the blocked kernels (unclean, a cycle, rows of more than 16 entries,
    values that reach the top bit): every result is the oracle's and lands at its own index;
    RBG_MODE_NO_DAG gives the same results on the blocked path."""
    from redblackgraph_gb300 import synth, _lib
    rng = np.random.default_rng(11)
    ped = synth.pedigree(200, 9, 3, dtype=np.int64)
    p = rng.permutation(200)
    both = ped[p][:, p]                                              # both sides of the diagonal
    unclean = ped.copy()
    unclean[150, 3] = -7
    cyc = synth.pedigree(120, 8, 4, dtype=np.int64)
    Wc, _, _, _ = O.warshall(cyc)
    v, u = max(zip(*np.nonzero(np.tril(Wc, -1))), key=lambda t: t[0] - t[1])
    cyc[u, v] = 2
    wide = _random_dag(rng, 80, 0.05)
    wide[70, :40] = rng.integers(2, 4, size=40)                      # a row of 40 parents
    deep = np.zeros((40, 40), np.int64)
    np.fill_diagonal(deep, 1)
    for i in range(1, 40):
        deep[i, i - 1] = 3                                           # a chain: products past 31 bits
    mats = [ped, both, _random_dag(rng, 50, 0.1), unclean, cyc, wide, synth.pedigree(64, 6, 8), deep,
            synth.pedigree(90, 7, 5)[::-1, ::-1]]
    mats = [m.astype(np.int32) for m in mats]
    Ws, res = run_batch(mats)
    for A, W, r in zip(mats, Ws, res):
        Wo, do, so, _ = O.warshall(A)
        assert r.status == so
        if so == 0:
            assert (W == Wo).all() and r.diameter == do
    paths = [r.path for r in res]
    dag, blk = _lib.PATH_DAG, _lib.PATH_BLOCKED32
    assert [paths[k] for k in (0, 1, 2, 3, 5, 6, 7, 8)] == [dag, dag, dag, _lib.PATH_EXACT, blk, dag,
                                                           paths[7], dag], paths
    assert res[4].status == _lib.RBG_ERR_CYCLE and paths[4] != dag and paths[7] != dag
    Ws2, res2 = run_batch(mats, mode=_lib.MODE_NO_DAG)
    for W, W2, r, r2 in zip(Ws, Ws2, res, res2):
        assert r2.status == r.status and r2.path != _lib.PATH_DAG
        if r.status == 0:
            assert (W == W2).all() and r.diameter == r2.diameter


def test_dag_path_graph_release(native):
    """rbg_release_scratch frees the DAG path's cached CUDA graphs; the next call records again
    and gives the same results."""
    from redblackgraph_gb300 import synth, _lib
    mats = [synth.pedigree(n, 9, n, dtype=np.int32) for n in (40, 300, 900)]
    Ws, res = run_batch(mats, mode=_lib.MODE_GRAPH)
    assert all(r.path == _lib.PATH_DAG for r in res)
    _lib.check(_lib.load().rbg_release_scratch(), "release_scratch")
    _lib.check(_lib.load().rbg_release_scratch(), "release_scratch")     # twice is harmless
    Ws2, res2 = run_batch(mats, mode=_lib.MODE_GRAPH)
    for W, W2, r, r2 in zip(Ws, Ws2, res, res2):
        assert (W == W2).all() and r.diameter == r2.diameter and r2.path == _lib.PATH_DAG


def test_dag_path_int64_mixed_batch(native):
    """int64 storage: pedigrees take the DAG path; values past 31 bits (in the input or in a
    product) send their matrix to the blocked kernels with 64-bit lanes; every result is the
    oracle's."""
    from redblackgraph_gb300 import synth, _lib
    ped = synth.pedigree(400, 14, 21, dtype=np.int64)
    big_in = ped.copy()
    big_in[399, 0] = 1 << 40                                         # an input value past 31 bits
    deep = np.zeros((45, 45), np.int64)
    np.fill_diagonal(deep, -1)
    for i in range(1, 45):
        deep[i, i - 1] = 2                                           # products reach bit 44
    mats = [ped, big_in, deep, synth.pedigree(64, 6, 8, dtype=np.int64)[::-1, ::-1].copy()]
    Ws, res = run_batch(mats)
    for A, W, r in zip(mats, Ws, res):
        Wo, do, so, _ = O.warshall(A)
        assert r.status == so == 0
        assert (W == Wo).all() and r.diameter == do
    assert [r.path for r in res] == [_lib.PATH_DAG, _lib.PATH_BLOCKED64, _lib.PATH_BLOCKED64, _lib.PATH_DAG]


def test_dag_path_calls_on_two_streams_overlap(native):
    """Two DAG-path batches on two streams from two host threads run at the same time: nothing in
    the library serialises calls.  Stream 1 first spins for ~150 ms, then closes batch A; while
    thread 1 waits inside its call, thread 2 closes batch B on stream 2.  B's last event must
    come before the end of stream 1's spin (so before A even started), and both results equal
    the oracle's.  Each thread first closes its batch once, so that its workspace and output
    exist: a device allocation during the measured calls would itself order the two streams."""
    import threading
    import time
    import torch
    from redblackgraph_gb300 import synth, _lib
    from redblackgraph_gb300.dense import fw_batch, pack
    from redblackgraph_gb300.device import to_device, to_host
    mats_a = [synth.pedigree(n, 10, n, dtype=np.int32) for n in (300, 900, 1400)]
    mats_b = [synth.pedigree(n, 9, n + 1, dtype=np.int32) for n in (250, 700)]
    fa, sa, oa = pack(mats_a)
    fb, sb, ob = pack(mats_b)
    da, db = to_device(fa), to_device(fb)
    outa, outb = torch.empty_like(da), torch.empty_like(db)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    spin_end = torch.cuda.Event(enable_timing=True)
    b_end = torch.cuda.Event(enable_timing=True)
    warm_a, warm_b, entered = threading.Event(), threading.Event(), threading.Event()
    out = {}

    def first():
        with torch.cuda.stream(s1):
            fw_batch(da, sa, oa, out=outa, stream=s1)      # this thread's workspace
            warm_a.set()
            warm_b.wait(30)
            torch.cuda._sleep(int(1.5e8 * 2))              # ~150 ms at 2 GHz: bounded spin
            spin_end.record(s1)
            entered.set()
            out["a"] = fw_batch(da, sa, oa, out=outa, stream=s1)

    def second():
        warm_a.wait(30)
        with torch.cuda.stream(s2):
            fw_batch(db, sb, ob, out=outb, stream=s2)
        warm_b.set()
        entered.wait(30)
        time.sleep(0.01)                                   # thread 1 is inside its call by now
        with torch.cuda.stream(s2):
            out["b"] = fw_batch(db, sb, ob, out=outb, stream=s2)
            b_end.record(s2)

    t1, t2 = threading.Thread(target=first), threading.Thread(target=second)
    t1.start()
    t2.start()
    t2.join(60)
    t1.join(60)
    torch.cuda.synchronize()
    assert spin_end.elapsed_time(b_end) < 0, "batch B waited for batch A"
    for mats, (o, res), offs, sizes in ((mats_a, out["a"], oa, sa), (mats_b, out["b"], ob, sb)):
        h = to_host(o)
        for A, r, k, n in zip(mats, res, offs, sizes):
            Wo, do, so, _ = O.warshall(A)
            assert r.path == _lib.PATH_DAG and r.status == so == 0 and r.diameter == do
            assert (h[k:k + n * n].reshape(n, n) == Wo).all()


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_dag_path_any_numbering_vs_oracle(native, dtype):
    """Matrices whose vertices are not numbered in a topological order (random relabellings of
    DAGs and pedigrees, entries on both sides of the diagonal) take the DAG path: the sequential
    loop replayed on the closure's pattern gives the oracle's values, diameters (each cell's
    first value in loop order) and errors, in both semantics (Cython: int32); deep ones whose
    products reach bit 31, and cyclic ones, leave the path with the oracle's results."""
    from redblackgraph_gb300 import synth, _lib
    rng = np.random.default_rng(23)
    mats = []
    for t in range(70):
        n = int(rng.integers(2, 80))
        A = _random_dag(rng, n, rng.uniform(0.03, 0.35))
        p = rng.permutation(n)
        mats.append(A[p][:, p].astype(dtype))
    # (the last one's closure pattern, ~64,000 cells, is past what one CTA replays in shared memory)
    for n, gens in ((120, None), (600, None), (1500, None), (2000, None), (2000, 100)):
        A = synth.pedigree(n, gens or synth.generations_for(n), n + 5, dtype=dtype)
        p = rng.permutation(n)
        mats.append(A[p][:, p].copy())
    cyc = synth.pedigree(150, 8, 41, dtype=dtype)
    Wc, _, _, _ = O.warshall(cyc)
    v, u = max(zip(*np.nonzero(np.tril(Wc, -1))), key=lambda t: t[0] - t[1])
    cyc[u, v] = 2
    p = rng.permutation(150)
    mats.append(cyc[p][:, p].copy())
    semantics = ((0, O.warshall), (_lib.MODE_CYTHON, O.fw_cython)) if dtype == np.int32 else ((0, O.warshall),)
    for mode, oracle in semantics:
        expect = [oracle(A) for A in mats]
        for graph in (0, _lib.MODE_GRAPH):
            Ws, res = run_batch(mats, mode=mode | graph)
            dag = 0
            for A, W, r, (Wo, do, so, _) in zip(mats, Ws, res, expect):
                assert r.status == so
                if so == 0:
                    assert (W == Wo).all() and r.diameter == do
                dag += r.path == _lib.PATH_DAG
            assert dag >= 50
            assert res[-1].status == _lib.RBG_ERR_CYCLE and res[-1].path != _lib.PATH_DAG
            assert all(r.path == _lib.PATH_DAG for r in res[-6:-1])   # the relabelled pedigrees
