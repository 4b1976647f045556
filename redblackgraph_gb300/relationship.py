"""Relationship lookups on closed red/black graphs, on the GPU.

``calculate_relationship(a, b)`` mirrors redblackgraph/reference/calc_relationship.py:54-71:
for two rows of a transitive closure the common ancestor is the first index minimising
``a[j] + b[j]`` among the indices where both rows are non-zero, and the relationship name
comes from the generational distances MSB(a[j]) and MSB(b[j]) (lookup_relationship,
:23-51).  The sums wrap in the rows' dtype, as the numpy scalars of the reference's rows do
(the unsigned red one, the dtype's maximum, plus y gives y - 1).  The search runs in
``rbg_relationship_lookup`` (one warp per query); ``lookup_many`` answers a whole batch of
(matrix, u, v) queries on resident device matrices in one launch.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _lib
from .device import numpy_dtype, require_cuda, stream_handle, to_device


@dataclass
class Relationship:
    """(common ancestor, name): redblackgraph/types/relationship.py:4-7."""
    common_ancestor: int
    relationship: str


def msb(x: int) -> int:
    """Bit position of the leading bit; 0 for x <= 1 (redblackgraph/reference/rbg_math.py:1-11)."""
    x = int(x)
    return x.bit_length() - 1 if x > 1 else 0


def _cousinth(generational: int) -> str:
    return {2: "1st cousin", 3: "2nd cousin", 4: "3rd cousin"}.get(generational,
                                                                    f"{generational - 1}th cousin")


def _grandparentith(removal: int) -> str:
    return {4: "2nd", 5: "3rd"}.get(removal, f"{removal - 2}th")


def relationship_name(da: int, db: int) -> str:
    """Name from the generational distances of u and v to their common ancestor
    (calc_relationship.py:23-51, including its rough edges)."""
    removal = abs(da - db)
    if da == 0 or db == 0:
        return {1: "parent", 2: "grandparent", 3: "great grandparent"}.get(
            removal, f"{_grandparentith(removal)} great grandparent")
    generational = min(da, db)
    if generational == 1 and removal == 0:
        return "sibling"
    if generational == 1 and removal == 1:
        return "aunt/uncle"
    if removal == 0:
        return _cousinth(generational)
    return f"{_cousinth(generational)} {removal} removed"


def decode(out: np.ndarray, dtypes) -> list[Relationship]:
    """Relationships from the raw (count, 3) lookup results and each query's matrix dtype."""
    res = []
    for k, dt in enumerate(dtypes):
        j = int(out[k, 0])
        if j == -2:
            raise IndexError("relationship query out of range")
        if j < 0:
            res.append(Relationship(-1, "No Relationship"))
            continue
        bits = out[k, 1:3].astype(np.int64)
        x, y = (bits.view(np.uint64) if np.dtype(dt).kind == "u" else bits).astype(object)
        res.append(Relationship(j, relationship_name(msb(x), msb(y))))
    return res


def lookup_table(table_dev: torch.Tensor, count: int, stream=None) -> np.ndarray:
    """Run the lookups described by a device array of ``count`` rbg_lookup_t; returns the raw
    (count, 3) int64 results on the host."""
    out = torch.empty((max(count, 1), 3), dtype=torch.int64, device=table_dev.device)
    L = _lib.load()
    _lib.check(L.rbg_relationship_lookup(count, table_dev.data_ptr(), out.data_ptr(), stream_handle(stream)),
               "relationship_lookup")
    return out[:count].cpu().numpy()


def lookup_many(queries, stream=None) -> list[Relationship]:
    """Answer many queries ``(W, u, v)`` (W a 2-D device tensor with contiguous rows, u and v two
    of its row indices) with one kernel launch."""
    queries = list(queries)
    if not queries:
        return []
    dev = queries[0][0].device
    table = (_lib.RbgLookup * len(queries))()
    dtypes = []
    for k, (W, u, v) in enumerate(queries):
        if W.ndim != 2 or not W.is_cuda or (W.shape[1] > 1 and W.stride(1) != 1):
            raise ValueError("queries take 2-D CUDA matrices with contiguous rows")
        if not (0 <= int(u) < W.shape[0] and 0 <= int(v) < W.shape[0]):
            raise IndexError(f"vertices ({u}, {v}) outside a matrix of {W.shape[0]} rows")
        dt = numpy_dtype(W.dtype)
        dtypes.append(dt)
        table[k] = _lib.RbgLookup(W.data_ptr(), W.stride(0), W.shape[0], W.shape[1], int(u), int(v),
                                  _lib.dtype_code(dt), 0)
    raw = np.frombuffer(table, dtype=np.uint8).copy()
    return decode(lookup_table(to_device(raw, dev), len(queries), stream), dtypes)


def calculate_relationship(a: Sequence[int], b: Sequence[int]) -> Relationship:
    """Relationship between u and v given their closure rows a and b (calc_relationship.py:54-71)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape or a.ndim != 1:
        raise ValueError("a and b must be rows of the same length")
    dt = np.result_type(a.dtype, b.dtype)
    if dt.kind not in "iu":
        dt = np.dtype(np.int64)
    if a.size == 0:
        return Relationship(-1, "No Relationship")
    W = to_device(np.ascontiguousarray(np.stack([a.astype(dt), b.astype(dt)])), require_cuda())
    return lookup_many([(W, 0, 1)])[0]
