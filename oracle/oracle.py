"""ctypes front-end of the CPU oracle (``avos_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` -- always as the checker or the timed CPU reference, never
on the product path.  Every function restates one reference routine; the C file cites the
reference file:line for each.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

RBG_OK, RBG_ERR_OVERFLOW, RBG_ERR_CYCLE = 0, 1, 2
EV_OVF_SIZE, EV_OVF_ONES, EV_HANG = 1, 2, 4

_SUFFIX = {
    np.dtype(np.int8): "i8", np.dtype(np.uint8): "u8",
    np.dtype(np.int16): "i16", np.dtype(np.uint16): "u16",
    np.dtype(np.int32): "i32", np.dtype(np.uint32): "u32",
    np.dtype(np.int64): "i64", np.dtype(np.uint64): "u64",
}
_CTYPE = {
    "i8": ctypes.c_int8, "u8": ctypes.c_uint8, "i16": ctypes.c_int16, "u16": ctypes.c_uint16,
    "i32": ctypes.c_int32, "u32": ctypes.c_uint32, "i64": ctypes.c_int64, "u64": ctypes.c_uint64,
}
_UCTYPE = {
    "i8": ctypes.c_uint8, "u8": ctypes.c_uint8, "i16": ctypes.c_uint16, "u16": ctypes.c_uint16,
    "i32": ctypes.c_uint32, "u32": ctypes.c_uint32, "i64": ctypes.c_uint64, "u64": ctypes.c_uint64,
}

_lib = None


def build() -> Path:
    """Compile the oracle with its Makefile (idempotent)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


def _declare(L):
    p = ctypes.c_void_p
    i64 = ctypes.c_int64
    for s in _SUFFIX.values():
        T, U = _CTYPE[s], _UCTYPE[s]
        getattr(L, f"orc_avos_sum_{s}").restype = T
        getattr(L, f"orc_avos_sum_{s}").argtypes = [T, T]
        getattr(L, f"orc_avos_product_{s}").restype = ctypes.c_int
        getattr(L, f"orc_avos_product_{s}").argtypes = [T, T, ctypes.POINTER(U)]
        getattr(L, f"orc_msb_{s}").restype = ctypes.c_int
        getattr(L, f"orc_msb_{s}").argtypes = [T]
        getattr(L, f"orc_warshall_{s}").restype = ctypes.c_int
        getattr(L, f"orc_warshall_{s}").argtypes = [i64, p, ctypes.c_int, p, p]
        getattr(L, f"orc_matmul_{s}").restype = ctypes.c_int
        getattr(L, f"orc_matmul_{s}").argtypes = [i64, i64, i64, p, p, p, p]
    L.orc_fw_cython_i32.restype = ctypes.c_int
    L.orc_fw_cython_i32.argtypes = [i64, p, ctypes.c_int, p, p]
    L.orc_cy_product.restype = ctypes.c_int32
    L.orc_cy_product.argtypes = [ctypes.c_int32, ctypes.c_int32]
    L.orc_cy_sum.restype = ctypes.c_int32
    L.orc_cy_sum.argtypes = [ctypes.c_int32, ctypes.c_int32]
    for s in _SUFFIX.values():
        T = _CTYPE[s]
        getattr(L, f"orc_vertex_comp_{s}").restype = ctypes.c_int
        getattr(L, f"orc_vertex_comp_{s}").argtypes = [i64, p, p, p, T, p, p]
        getattr(L, f"orc_edge_comp_{s}").restype = ctypes.c_int
        getattr(L, f"orc_edge_comp_{s}").argtypes = [i64, p, i64, i64, T, p, p]
    L.orc_vertex_comp_cy.restype = None
    L.orc_vertex_comp_cy.argtypes = [i64, p, p, p, ctypes.c_int32, p]
    L.orc_edge_comp_cy.restype = None
    L.orc_edge_comp_cy.argtypes = [i64, p, i64, i64, ctypes.c_int32, p]
    L.orc_spgemm_pass1.restype = i64
    L.orc_spgemm_pass1.argtypes = [i64, i64, p, p, p, p, p]
    for s in ("i64", "u64"):
        getattr(L, f"orc_spgemm_pass2_{s}").restype = i64
        getattr(L, f"orc_spgemm_pass2_{s}").argtypes = [i64, i64, p, p, p, p, p, p, p, p, p, p]


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def suffix(dtype) -> str:
    return _SUFFIX[np.dtype(dtype)]


# ----------------------------------------------------------------------------- scalars
def avos_sum(x, y, dtype=np.int64):
    s = suffix(dtype)
    T = _CTYPE[s]
    return getattr(lib(), f"orc_avos_sum_{s}")(T(int(x)).value, T(int(y)).value)


def avos_product(x, y, dtype=np.int64):
    """Return (unsigned result, event flags) of the C core's avos_product."""
    s = suffix(dtype)
    T, U = _CTYPE[s], _UCTYPE[s]
    out = U(0)
    ev = getattr(lib(), f"orc_avos_product_{s}")(T(int(x)).value, T(int(y)).value,
                                                  ctypes.byref(out))
    return out.value, ev


def cy_product(x, y):
    return lib().orc_cy_product(int(np.int32(x)), int(np.int32(y)))


def cy_sum(x, y):
    return lib().orc_cy_sum(int(np.int32(x)), int(np.int32(y)))


# ----------------------------------------------------------------------------- dense
def warshall(a: np.ndarray, triangular: bool = False):
    """C core ``warshall`` on one square matrix.

    Returns ``(W, diameter, status, info)``; ``status`` is 0, RBG_ERR_OVERFLOW or
    RBG_ERR_CYCLE (the exception the reference raises), ``info`` = [kind, flags, k, i, j].
    """
    w = np.ascontiguousarray(a).copy()
    n = w.shape[0]
    assert w.shape == (n, n)
    d = np.zeros(1, np.int64)
    info = np.zeros(5, np.int64)
    st = getattr(lib(), f"orc_warshall_{suffix(w.dtype)}")(n, _ptr(w), int(triangular),
                                                            _ptr(d), _ptr(info))
    return w, int(d[0]), int(st), info


def fw_cython(a: np.ndarray, triangular: bool = False):
    """Cython ``floyd_warshall`` (int32): returns ``(W, diameter, status, info)``."""
    w = np.ascontiguousarray(a, dtype=np.int32).copy()
    n = w.shape[0]
    d = np.zeros(1, np.int64)
    info = np.zeros(4, np.int64)
    st = lib().orc_fw_cython_i32(n, _ptr(w), int(triangular), _ptr(d), _ptr(info))
    return w, int(d[0]), int(st), info


def matmul(a: np.ndarray, b: np.ndarray):
    """Dense AVOS product ``a @ b`` (C core einsum 'ij,jk'); returns ``(C, status, flags)``."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    m, q = a.shape
    q2, p = b.shape
    assert q == q2
    c = np.zeros((m, p), a.dtype)
    fl = np.zeros(1, np.int64)
    st = getattr(lib(), f"orc_matmul_{suffix(a.dtype)}")(m, q, p, _ptr(a), _ptr(b), _ptr(c),
                                                         _ptr(fl))
    return c, int(st), int(fl[0])


# ----------------------------------------------------------------------------- sparse
def spgemm(indptr_a, indices_a, data_a, indptr_b, indices_b, data_b, n_row, n_col):
    """rbm_matmat_pass1 + pass2 on 64-bit values and int64 indices.

    Inputs must be canonical CSR (sorted, no duplicates), data already 64-bit.
    Returns ``(indptr, indices, data, flags)`` with columns in the reference's
    accumulator order.
    """
    ap = np.ascontiguousarray(indptr_a, np.int64)
    aj = np.ascontiguousarray(indices_a, np.int64)
    bp = np.ascontiguousarray(indptr_b, np.int64)
    bj = np.ascontiguousarray(indices_b, np.int64)
    ax = np.ascontiguousarray(data_a)
    bx = np.ascontiguousarray(data_b, ax.dtype)
    s = suffix(ax.dtype)
    assert s in ("i64", "u64")
    cp = np.zeros(n_row + 1, np.int64)
    nnz = lib().orc_spgemm_pass1(n_row, n_col, _ptr(ap), _ptr(aj), _ptr(bp), _ptr(bj), _ptr(cp))
    cj = np.zeros(max(nnz, 1), np.int64)
    cx = np.zeros(max(nnz, 1), ax.dtype)
    fl = np.zeros(1, np.int64)
    nnz2 = getattr(lib(), f"orc_spgemm_pass2_{s}")(n_row, n_col, _ptr(ap), _ptr(aj), _ptr(ax),
                                                   _ptr(bp), _ptr(bj), _ptr(bx), _ptr(cp),
                                                   _ptr(cj), _ptr(cx), _ptr(fl))
    return cp, cj[:nnz2], cx[:nnz2], int(fl[0])


def rb_matmul_csr(a, b):
    """``rb_matrix.__matmul__`` (rbm.py:39-122) on scipy CSR inputs: canonicalise,
    upcast values to 64 bits (with the unsigned RED_ONE remap), pass 1/2, cast back.
    Returns a scipy ``csr_matrix`` and the product event flags."""
    import scipy.sparse as sp
    a = sp.csr_matrix(a, copy=True)
    b = sp.csr_matrix(b, copy=True)
    for m in (a, b):
        m.sort_indices()
        m.sum_duplicates()
    out_dtype = np.promote_types(a.dtype, b.dtype)
    wide = np.dtype(np.uint64) if out_dtype.kind == "u" else np.dtype(np.int64)

    def widen(m):
        d = np.asarray(m.data).astype(wide)
        if out_dtype.kind == "u" and m.data.dtype.itemsize < 8:
            d[m.data == np.iinfo(m.data.dtype).max] = np.iinfo(wide).max
        return d

    cp, cj, cx, fl = spgemm(a.indptr, a.indices, widen(a), b.indptr, b.indices, widen(b),
                            a.shape[0], b.shape[1])
    res = sp.csr_matrix((cx.astype(out_dtype), cj, cp), shape=(a.shape[0], b.shape[1]))
    return res, fl


def components(indptr, indices, n: int) -> np.ndarray:
    """Weakly connected components numbered by their least vertex (find_components_sparse,
    redblackgraph/sparse/csgraph/_components.pyx:86-177: a DFS started from each unvisited
    vertex in increasing order, following edges both ways).  Label propagation in numpy."""
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(np.asarray(indptr, dtype=np.int64)))
    cols = np.asarray(indices, dtype=np.int64)
    lab = np.arange(n, dtype=np.int64)
    while True:
        m = np.minimum(lab[rows], lab[cols])
        new = lab.copy()
        np.minimum.at(new, rows, m)
        np.minimum.at(new, cols, m)
        new = new[new]                          # pointer jumping
        if (new == lab).all():
            break
        lab = new
    roots = np.unique(lab)                      # ascending = ordered by least vertex
    return np.searchsorted(roots, lab).astype(np.int64)


def component_wise_closure(a, method: str = "auto", densify_threshold: int = 500):
    """component_wise_closure (redblackgraph/sparse/csgraph/transitive_closure.py:85-195) with
    each component closed by the Cython Floyd-Warshall restatement.

    Returns ``(W csr int32, diameter, None)`` or ``(None, None, (component, info))`` for the first
    component (by number) whose closure raises CycleError; ``info`` holds the local [kind, k, i, j].
    A component takes the Floyd-Warshall diameter (running maximum) when the reference would
    close it with floyd_warshall (:172-176) and MSB of its largest final value otherwise (:178-182,
    _shortest_path.pyx:842-845); a single component takes "FW" only when asked (:151-158).
    """
    import scipy.sparse as sp
    csr = sp.csr_matrix(a, copy=True)
    csr.sum_duplicates()
    csr.sort_indices()
    n = csr.shape[0]
    if n == 0:
        return sp.csr_matrix((0, 0), dtype=np.int32), 0, None
    lab = components(csr.indptr, csr.indices, n)
    k = int(lab.max()) + 1
    rows, cols, vals = [], [], []
    diameter = 0
    for c in range(k):
        verts = np.flatnonzero(lab == c)
        sub = csr[verts][:, verts].toarray().astype(np.int32)
        W, d, st, info = fw_cython(sub)
        if st != 0:
            return None, None, (c, info)
        fw = (method == "FW") if k == 1 else (len(verts) <= densify_threshold if method == "auto"
                                              else method == "FW")
        if not fw:
            mx = int(W.max())
            d = mx.bit_length() - 1 if mx > 1 else 0
        diameter = max(diameter, d)
        r, cc = np.nonzero(W)
        rows.append(verts[r])
        cols.append(verts[cc])
        vals.append(W[r, cc])
    W = sp.csr_matrix((np.concatenate(vals).astype(np.int32),
                       (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    W.sort_indices()
    return W, diameter, None


def _wrap(v: int, dtype) -> int:
    """v reduced to the range of the integer dtype (two's complement wrap)."""
    info = np.iinfo(dtype)
    span = 1 << (8 * np.dtype(dtype).itemsize)
    return (v - int(info.min)) % span + int(info.min)


def calculate_relationship(a, b):
    """calculate_relationship (redblackgraph/reference/calc_relationship.py:54-71) on two closure
    rows given as numpy arrays: the first j minimising a[j] + b[j] over the j where both are
    non-zero, the sum taken as numpy scalar arithmetic does (wrapping in the rows' dtype);
    then the name from MSB of the two values (rbg_math.py:1-11, calc_relationship.py:23-51).
    Returns (common ancestor, name)."""
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.result_type(a.dtype, b.dtype)
    best, bj = None, -1
    for j in range(a.size):
        x, y = int(a[j]), int(b[j])
        if x != 0 and y != 0:
            s = _wrap(x + y, dt)
            if best is None or s < best:
                best, bj = s, j
    if bj < 0:
        return -1, "No Relationship"

    def msb(x):
        p = 0
        while x > 1:
            x >>= 1
            p += 1
        return p

    da, db = msb(int(a[bj])), msb(int(b[bj]))
    removal = abs(da - db)

    def cousinth(g):
        return {2: "1st cousin", 3: "2nd cousin", 4: "3rd cousin"}.get(g, f"{g - 1}th cousin")

    if da == 0 or db == 0:
        names = {1: "parent", 2: "grandparent", 3: "great grandparent"}
        if removal in names:
            return bj, names[removal]
        gp = {4: "2nd", 5: "3rd"}.get(removal, f"{removal - 2}th")
        return bj, f"{gp} great grandparent"
    g = min(da, db)
    if g == 1 and removal == 0:
        return bj, "sibling"
    if g == 1 and removal == 1:
        return bj, "aunt/uncle"
    if removal == 0:
        return bj, cousinth(g)
    return bj, f"{cousinth(g)} {removal} removed"


def _cy_msb(x: int) -> int:
    p = 0
    while x > 1:
        x >>= 1
        p += 1
    return p


def _i32(v: int) -> int:
    v &= 0xffffffff
    return v - (1 << 32) if v >= (1 << 31) else v


def cy_product_py(lhs: int, rhs: int) -> int:
    """The Cython avos_product on int32 (redblackgraph/sparse/csgraph/_rbg_math.pxi:33-87)."""
    x, y = lhs & 0xffffffff, rhs & 0xffffffff
    if x == 0 or y == 0:
        return 0
    if lhs == -1 and rhs == -1:
        return -1
    if lhs == 1 and rhs == 1:
        return 1
    if (lhs == -1 and rhs == 1) or (lhs == 1 and rhs == -1):
        return 0
    if lhs == -1:
        x = 1
    if rhs == -1:
        return 0 if lhs & 1 else _i32(x)
    if rhs == 1:
        return _i32(x) if lhs & 1 else 0
    bp = _cy_msb(_i32(y))
    low = 0 if bp == 0 else (y & ((1 << bp) - 1))
    return _i32(low | (x << bp))


def cy_sum_py(x: int, y: int) -> int:
    """The Cython avos_sum on int32 (_rbg_math.pxi:18-31): the non-zero minimum, signed."""
    if x == 0:
        return y
    if y == 0:
        return x
    return x if x < y else y


def dag_closure(a):
    """transitive_closure_dag_sparse_cython (redblackgraph/sparse/csgraph/_transitive_closure_dag.pyx:
    168-351), restated for small graphs: rows built parents first, each parent's closed row
    multiplied in by the edge value, candidates folded with the Cython sum; the diameter is MSB of
    the largest magnitude of any stored entry or candidate.  Returns ``(W csr int32, diameter)``;
    raises ValueError on a cycle."""
    import scipy.sparse as sp
    A = sp.csr_matrix(a)
    A.sum_duplicates()
    A.sort_indices()
    n = A.shape[0]
    ip, ij = A.indptr, A.indices
    dv = np.asarray(A.data).astype(np.int64)
    dv = np.array([_i32(int(v)) for v in dv], dtype=np.int64)
    # parents first: Kahn's order on the edges v -> w (w != v)
    deg = np.zeros(n, dtype=np.int64)
    children = [[] for _ in range(n)]
    for v in range(n):
        for e in range(ip[v], ip[v + 1]):
            w = int(ij[e])
            if w != v:
                deg[v] += 1
                children[w].append(v)
    order, ready = [], [v for v in range(n) if deg[v] == 0]
    while ready:
        w = ready.pop()
        order.append(w)
        for v in children[w]:
            deg[v] -= 1
            if deg[v] == 0:
                ready.append(v)
    if len(order) != n:
        raise ValueError("graph contains a cycle")
    rows = [None] * n
    mx = 0
    for v in order:
        row = {}
        for e in range(ip[v], ip[v + 1]):
            w, val = int(ij[e]), int(dv[e])
            row[w] = cy_sum_py(row[w], val) if w in row else val
            mx = max(mx, abs(val) if val != -(1 << 31) else 0)
        for e in range(ip[v], ip[v + 1]):
            w, a_vw = int(ij[e]), int(dv[e])
            if w == v:
                continue
            for x, c in rows[w].items():
                p = cy_product_py(a_vw, c)
                if p == 0:
                    continue
                row[x] = cy_sum_py(row[x], p) if x in row else p
                mx = max(mx, abs(p) if p != -(1 << 31) else 0)
        rows[v] = row
    r_, c_, v_ = [], [], []
    for v in range(n):
        for x in sorted(rows[v]):
            r_.append(v)
            c_.append(x)
            v_.append(rows[v][x])
    W = sp.csr_matrix((np.array(v_, dtype=np.int32), (np.array(r_, dtype=np.int64), np.array(c_, dtype=np.int64))),
                      shape=(n, n))
    W.sort_indices()
    return W, (_cy_msb(mx) if mx > 1 else 0)


# ----------------------------------------------------------------------------- composition
def vertex_compose(R, u, v, color):
    """C core vertex relational composition (relational_composition.c.in:166-262) in the
    reference's loop order.  Returns ``(out, info)``; info = [status, flags, step, i, j, lhs,
    rhs, event] of the deciding event (status 0 when none)."""
    R = np.ascontiguousarray(R)
    dt = R.dtype
    n = R.shape[0]
    u = np.ascontiguousarray(np.asarray(u).reshape(-1), dtype=dt)
    v = np.ascontiguousarray(np.asarray(v).reshape(-1), dtype=dt)
    out = np.zeros((n + 1, n + 1), dtype=dt)
    info = np.zeros(8, dtype=np.int64)
    s = suffix(dt)
    c = _CTYPE[s](int(np.array(color).astype(dt))).value
    getattr(lib(), f"orc_vertex_comp_{s}")(n, _ptr(R), _ptr(u), _ptr(v), c, _ptr(out), _ptr(info))
    return out, info


def edge_compose(R, alpha, beta, relationship):
    """C core edge relational composition (relational_composition.c.in:72-139)."""
    R = np.ascontiguousarray(R)
    dt = R.dtype
    n = R.shape[0]
    out = np.zeros((n, n), dtype=dt)
    info = np.zeros(8, dtype=np.int64)
    s = suffix(dt)
    r = _CTYPE[s](int(np.array(relationship).astype(dt))).value
    getattr(lib(), f"orc_edge_comp_{s}")(n, _ptr(R), int(alpha), int(beta), r, _ptr(out), _ptr(info))
    return out, info


def vertex_compose_cy(R, u, v, color):
    """Cython vertex_relational_composition (_relational_composition.pyx:10-64), int32."""
    R = np.ascontiguousarray(R, dtype=np.int32)
    n = R.shape[0]
    u = np.ascontiguousarray(np.asarray(u).reshape(-1), dtype=np.int32)
    v = np.ascontiguousarray(np.asarray(v).reshape(-1), dtype=np.int32)
    out = np.zeros((n + 1, n + 1), dtype=np.int32)
    lib().orc_vertex_comp_cy(n, _ptr(R), _ptr(u), _ptr(v), int(np.int32(color)), _ptr(out))
    return out


def edge_compose_cy(R, alpha, beta, relationship):
    """Cython edge_relational_composition (_relational_composition.pyx:67-113), int32."""
    R = np.ascontiguousarray(R, dtype=np.int32)
    n = R.shape[0]
    out = np.zeros((n, n), dtype=np.int32)
    lib().orc_edge_comp_cy(n, _ptr(R), int(alpha), int(beta), int(np.int32(relationship)), _ptr(out))
    return out


# ----------------------------------------------------------------------------- orderings
def ordering_metrics(A):
    """Per vertex (ancestor count, column maximum, diagonal) as _get_permutation /
    _compute_ordering_metrics_sparse compute them (_ordering.pyx:15-39, 101-149)."""
    import scipy.sparse as sp
    if sp.issparse(A):
        csr = sp.csr_matrix(A)
        n = csr.shape[0]
        anc = np.zeros(n, np.int64)
        mx = np.zeros(n, np.int64)
        dg = np.zeros(n, np.int64)
        for i in range(n):
            for e in range(csr.indptr[i], csr.indptr[i + 1]):
                c, v = int(csr.indices[e]), int(np.int32(csr.data[e]))
                if v != 0:
                    anc[i] += _cy_msb(v)
                    mx[c] = max(mx[c], v)
                if c == i:
                    dg[i] = v
        return anc, mx, dg
    a = np.asarray(A).astype(np.int64)
    n = a.shape[0]
    anc = np.array([sum(_cy_msb(int(v)) for v in a[i] if v != 0) for i in range(n)], np.int64)
    mx = np.array([max([0] + [int(v) for v in a[:, i] if v != 0]) for i in range(n)], np.int64)
    return anc, mx, np.diag(a).copy()


def canonical_permutation(A, q, ids):
    """The canonical order's sort (_ordering.pyx:37-38, 92-97)."""
    anc, mx, dg = ordering_metrics(A)
    ids = np.asarray(ids)
    return sorted(range(len(ids)), key=lambda x: (-q[int(ids[x])], int(ids[x]), -anc[x], mx[x], -dg[x], x))


def permute_dense(A, p, upper=False):
    """B[i][j] = A[p[i]][p[j]], j >= i when triangular (_permutation.pyx:48-63)."""
    a = np.asarray(A)
    n = a.shape[0]
    B = np.zeros((n, n), np.int32)
    for i in range(n):
        for j in range(i if upper else 0, n):
            B[i, j] = a[p[i], p[j]]
    return B


def topological_sort_dfs(A):
    """The reference's iterative depth-first topological sort (_topological_sort.pyx:30-181):
    reverse post-order from every unvisited vertex in order, neighbours in CSR order, diagonal
    skipped; ValueError on a back edge."""
    import scipy.sparse as sp
    csr = sp.csr_matrix(A)
    n = csr.shape[0]
    ip, ij = csr.indptr, csr.indices
    color = [0] * n
    order = [0] * n
    at = n - 1
    for s in range(n):
        if color[s]:
            continue
        stack = [[s, ip[s]]]
        color[s] = 1
        while stack:
            v, idx = stack[-1]
            pushed = False
            while idx < ip[v + 1]:
                w = int(ij[idx])
                idx += 1
                if w == v:
                    continue
                if color[w] == 0:
                    stack[-1][1] = idx
                    stack.append([w, ip[w]])
                    color[w] = 1
                    pushed = True
                    break
                if color[w] == 1:
                    raise ValueError(f"cycle at {w}")
            if not pushed:
                color[v] = 2
                order[at] = v
                at -= 1
                stack.pop()
    return np.array(order, np.int32)
