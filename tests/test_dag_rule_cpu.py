"""The rule behind the DAG path, checked on the CPU against the oracle's sequential loop.

For a matrix whose off-diagonal entries all lie below (or all above) the diagonal, the
sequential Floyd-Warshall loop equals the DAG recurrence, and its diameter (the largest value
ever written) is the largest first value of any cell: A(i, j), else the product of the first step
that reaches the cell (below: the smallest parent k of i with j in C(k); above: the smallest k in
C(i) with j a parent of k).  This restates that rule in plain Python (the GPU kernels implement
it in fw_tri.cu / dag_rows.cuh) and compares it with the oracle on random DAGs, a third of which
have a diameter above their final values' MSB."""
import numpy as np

from oracle import oracle as O


def _msb(x):
    return int(x).bit_length() - 1


def _prod(x, y):
    b = _msb(y)
    return (x << b) | (y & ((1 << b) - 1))


def _dag_rule(A):
    n = A.shape[0]
    par = {i: [j for j in range(n) if j != i and A[i, j] != 0] for i in range(n)}
    above = any(j > i for i in range(n) for j in par[i])
    C = {}
    for i in (range(n - 1, -1, -1) if above else range(n)):
        row = {j: int(A[i, j]) for j in par[i]}
        for k in par[i]:
            for j, v in C[k].items():
                p = _prod(int(A[i, k]), v)
                row[j] = min(row.get(j, p), p)
        C[i] = row
    top, first = -1, -1
    for i in range(n):
        seen = set(par[i])
        first = max([first] + [_msb(A[i, j]) for j in par[i]])
        for k in par[i]:                     # the recurrence's own candidates
            for v in C[k].values():
                top = max(top, _msb(A[i, k]) + _msb(v))
        steps = ([(k, C[k].items(), _msb(A[i, k]), True) for k in par[i]] if not above else
                 [(k, [(j, int(A[k, j])) for j in par[k]], _msb(C[i][k]), False) for k in sorted(C[i])])
        for k, items, mk, _ in steps:
            for j, v in sorted(items):
                pm = mk + _msb(v)
                top = max(top, pm)
                if j not in seen:
                    first = max(first, pm)
                    seen.add(j)
    W = A.copy()
    for i in range(n):
        for j, v in C[i].items():
            W[i, j] = v
    return W, max(first, 0), top


def test_dag_rule_matches_the_sequential_loop():
    rng = np.random.default_rng(1)
    checked = differs = 0
    for t in range(240):
        n = int(rng.integers(1, 32))
        A = np.zeros((n, n), np.int64)
        low = np.tril(rng.random((n, n)) < rng.uniform(0.02, 0.5), -1)
        A[low] = rng.integers(2, 8, size=int(low.sum()))
        np.fill_diagonal(A, rng.choice([-1, 0, 1], size=n))
        if t % 2:
            A = A[::-1, ::-1].copy()
        W, d, top = _dag_rule(A)
        if top >= 31:                        # the GPU path hands these to the blocked kernels
            continue
        Wo, do, so, _ = O.warshall(A.astype(np.int32))
        assert so == 0 and (W == Wo).all() and d == do, t
        checked += 1
        final = _msb(W[W > 1].max()) if (W > 1).any() else 0
        differs += d != final
    assert checked > 200 and differs > 30


def test_dag_rule_matches_the_reference_itself():
    """The same rule against the reference's own C warshall (where the reference is mounted and
    built: not on the GPU host)."""
    import pytest
    from oracle import refimport
    if not refimport.available():
        pytest.skip("reference not available here")
    refimport.load()
    import redblackgraph.core as core
    from redblackgraph.core.redblack import array as rb_array
    rng = np.random.default_rng(7)
    checked = 0
    for t in range(60):
        n = int(rng.integers(2, 28))
        A = np.zeros((n, n), np.int64)
        low = np.tril(rng.random((n, n)) < rng.uniform(0.05, 0.4), -1)
        A[low] = rng.integers(2, 8, size=int(low.sum()))
        np.fill_diagonal(A, rng.choice([-1, 1], size=n))
        if t % 2:
            A = A[::-1, ::-1].copy()
        W, d, top = _dag_rule(A)
        if top >= 31:
            continue
        A32 = A.astype(np.int32)
        Wr, dr = core.warshall(np.stack([A32, A32]).view(rb_array))
        assert (np.asarray(Wr[0]) == W).all() and int(np.asarray(dr).reshape(-1)[0]) == d, t
        checked += 1
    assert checked > 40


def _replay_on_pattern(A):
    """The sequential loop replayed only on the final closure's pattern (reachability), with the
    evolving values: for step k, the rows whose final pattern holds column k, merged with row k's
    current non-zeros.  Returns (W, diameter, largest product MSB)."""
    n = A.shape[0]
    reach = [set(j for j in range(n) if j != i and A[i, j] != 0) for i in range(n)]
    changed = True
    while changed:                                    # the pattern: plain reachability
        changed = False
        for i in range(n):
            new = set().union(*(reach[k] for k in reach[i])) - reach[i] - {i} if reach[i] else set()
            if new:
                reach[i] |= new
                changed = True
    col = [[i for i in range(n) if k in reach[i]] for k in range(n)]
    cur = {i: {j: int(A[i, j]) for j in reach[i] if A[i, j] != 0} for i in range(n)}
    first = max([_msb(v) for i in range(n) for v in cur[i].values()] + [-1])
    top = -1
    for k in range(n):
        rowk = list(cur[k].items())
        for i in col[k]:
            x = cur[i].get(k, 0)
            if x == 0:
                continue
            for j, y in rowk:
                if j == i:
                    continue
                p = _prod(x, y)
                top = max(top, _msb(p))
                old = cur[i].get(j, 0)
                if old == 0:
                    first = max(first, _msb(p))
                    cur[i][j] = p
                else:
                    cur[i][j] = min(old, p)
    W = A.copy()
    for i in range(n):
        for j, v in cur[i].items():
            W[i, j] = v
    return W, max(first, 0), top


def test_replay_on_the_pattern_matches_in_any_numbering():
    """For components numbered in any order (the plan for the ones the DAG path does not take):
    the loop replayed on the final pattern gives the oracle's values and diameter."""
    rng = np.random.default_rng(3)
    checked = 0
    for t in range(120):
        n = int(rng.integers(2, 26))
        A = np.zeros((n, n), np.int64)
        low = np.tril(rng.random((n, n)) < rng.uniform(0.05, 0.4), -1)
        A[low] = rng.integers(2, 8, size=int(low.sum()))
        np.fill_diagonal(A, rng.choice([-1, 0, 1], size=n))
        p = rng.permutation(n)
        A = A[p][:, p]                                # any numbering
        W, d, top = _replay_on_pattern(A)
        if top >= 31:
            continue
        Wo, do, so, _ = O.warshall(A.astype(np.int32))
        assert so == 0 and (W == Wo).all() and d == do, t
        checked += 1
    assert checked > 80
