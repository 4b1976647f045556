"""Seeded synthetic pedigrees (the bench and test inputs).

A pedigree is a red/black graph: row = child, column = parent (the reference's orientation,
redblackgraph/util/synthesizer.py:481-509).  Vertices are numbered oldest generation first, so
every parent edge points to a lower index and the matrix is lower triangular.  Each vertex is
red (male, diagonal -1) or black (female, diagonal 1) with probability 1/2; from generation 1
on it takes a father (value 2) with probability ``p_parent`` drawn uniformly among the males of
all earlier generations, and a mother (value 3) likewise among the females.

Forests (``forest``) are disjoint families laid out one after another; within a family the
parents come from the previous ``reach`` generations, which keeps ancestor sets small the way
real family trees are.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _generation_sizes(n: int, generations: int) -> np.ndarray:
    g = max(1, min(generations, n))
    sizes = np.full(g, n // g, dtype=np.int64)
    sizes[: n % g] += 1
    return sizes


def pedigree_edges(n: int, generations: int, seed: int, p_parent: float = 0.9):
    """Return (colors, child, parent, value) arrays of one pedigree component."""
    rng = np.random.default_rng(seed)
    colors = np.where(rng.random(n) < 0.5, -1, 1).astype(np.int64)
    sizes = _generation_sizes(n, generations)
    starts = np.concatenate([[0], np.cumsum(sizes)])
    gen_of = np.repeat(np.arange(len(sizes)), sizes)
    lo = starts[gen_of]                       # first vertex of each vertex's generation
    males = np.flatnonzero(colors == -1)
    females = np.flatnonzero(colors == 1)
    child, parent, value = [], [], []
    for pool, val in ((males, 2), (females, 3)):
        cnt = np.searchsorted(pool, lo)       # candidates strictly before the generation
        take = (rng.random(n) < p_parent) & (cnt > 0)
        idx = np.floor(rng.random(n) * np.maximum(cnt, 1)).astype(np.int64)
        v = np.flatnonzero(take)
        child.append(v)
        parent.append(pool[idx[v]])
        value.append(np.full(v.size, val, np.int64))
    return colors, np.concatenate(child), np.concatenate(parent), np.concatenate(value)


def pedigree(n: int, generations: int, seed: int, dtype=np.int32, p_parent: float = 0.9) -> np.ndarray:
    """Dense (n, n) pedigree matrix."""
    colors, c, p, v = pedigree_edges(n, generations, seed, p_parent)
    A = np.zeros((n, n), dtype=np.int64)
    A[np.arange(n), np.arange(n)] = colors
    A[c, p] = v
    return A.astype(dtype)


def pedigree_csr(n: int, generations: int, seed: int, dtype=np.int32, p_parent: float = 0.9):
    colors, c, p, v = pedigree_edges(n, generations, seed, p_parent)
    rows = np.concatenate([np.arange(n), c])
    cols = np.concatenate([np.arange(n), p])
    vals = np.concatenate([colors, v]).astype(dtype)
    m = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    m.sort_indices()
    return m


def component_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """Log-uniform integer sizes in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.clip(np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), count))), lo, hi).astype(np.int64)


def generations_for(n: int) -> int:
    """Generation depth proportional to log2(size)."""
    return int(max(2, round(1.5 * np.log2(max(n, 2)))))


def batch_components(count: int = 4096, lo: int = 16, hi: int = 4096, seed: int = 3, dtype=np.int32):
    """Sizes and per-component seeds of the batched-closure workload."""
    sizes = component_sizes(count, lo, hi, seed)
    seeds = (np.arange(count, dtype=np.int64) * 7919 + seed * 1_000_003) % (2**31 - 1)
    return sizes, seeds


def forest(n: int, generations: int, seed: int, family: int = 64, reach: int = 2,
           p_parent: float = 0.9, dtype=np.int64):
    """Sparse forest of disjoint pedigree families (CSR, int32 indices)."""
    rng = np.random.default_rng(seed)
    colors = np.where(rng.random(n) < 0.5, -1, 1).astype(np.int64)
    fam = np.arange(n) // family
    pos = np.arange(n) % family
    fsize = np.minimum(family, n - fam * family)
    gens = np.maximum(1, np.minimum(generations, fsize))
    gen = (pos * gens) // fsize                        # generation inside the family
    gstart = fam * family + (gen * fsize + gens - 1) // gens
    lo_gen = np.maximum(gen - reach, 0)
    lo = fam * family + (lo_gen * fsize + gens - 1) // gens
    rows, cols, vals = [np.arange(n)], [np.arange(n)], [colors]
    for want, val in ((-1, 2), (1, 3)):
        # draw candidates in [lo, gstart) until the colour matches (bounded tries)
        cand = np.full(n, -1, np.int64)
        span = gstart - lo
        for _ in range(8):
            r = lo + np.floor(rng.random(n) * np.maximum(span, 1)).astype(np.int64)
            ok = (span > 0) & (cand < 0) & (colors[np.minimum(r, n - 1)] == want)
            cand[ok] = r[ok]
        take = (rng.random(n) < p_parent) & (cand >= 0)
        v = np.flatnonzero(take)
        rows.append(v)
        cols.append(cand[v])
        vals.append(np.full(v.size, val, np.int64))
    m = sp.csr_matrix((np.concatenate(vals).astype(dtype),
                       (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    m.sort_indices()
    m.indices = m.indices.astype(np.int32)
    m.indptr = m.indptr.astype(np.int64 if m.nnz >= 2**31 else np.int32)
    return m


def batch_edges(sizes, seeds, p_parent: float = 0.9):
    """Edge lists of many pedigree components laid out one after another in a flat buffer of
    dense matrices: returns (flat_index, value, offsets) with flat_index into that buffer."""
    sizes = np.asarray(sizes, dtype=np.int64)
    offsets = np.zeros_like(sizes)
    if sizes.size > 1:
        offsets[1:] = np.cumsum(sizes[:-1] * sizes[:-1])
    idx, val = [], []
    for n, s, o in zip(sizes, seeds, offsets):
        n = int(n)
        colors, c, p, v = pedigree_edges(n, generations_for(n), int(s), p_parent)
        ar = np.arange(n, dtype=np.int64)
        idx.append(o + ar * n + ar)
        val.append(colors)
        idx.append(o + c * n + p)
        val.append(v)
    return np.concatenate(idx), np.concatenate(val), offsets


def batch_forest(sizes, seeds, p_parent: float = 0.9):
    """The pedigree components of ``batch_components`` laid out one after another as one sparse
    forest (block diagonal CSR, int32 values).  Component i is ``pedigree_csr(sizes[i],
    generations_for(sizes[i]), seeds[i])`` on vertices base[i] .. base[i] + sizes[i]."""
    sizes = np.asarray(sizes, dtype=np.int64)
    base = np.concatenate([[0], np.cumsum(sizes)])
    rows, cols, vals = [], [], []
    for n, s, b in zip(sizes, seeds, base[:-1]):
        n = int(n)
        colors, c, p, v = pedigree_edges(n, generations_for(n), int(s), p_parent)
        ar = np.arange(n, dtype=np.int64)
        rows += [b + ar, b + c]
        cols += [b + ar, b + p]
        vals += [colors, v]
    N = int(base[-1])
    m = sp.csr_matrix((np.concatenate(vals).astype(np.int32),
                       (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    m.sum_duplicates()
    m.sort_indices()
    return m, base
