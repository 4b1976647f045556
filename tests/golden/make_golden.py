"""Generate the golden fixtures by running the reference itself.

Run in a container where the reference tree is mounted and built (``python oracle/ref_build.py``):

    python tests/golden/make_golden.py

Every expected value below comes from calling the reference's own code (C core ``warshall``,
``rb.array @``, ``core.avos_sum/avos_product``, Cython ``floyd_warshall`` and
``transitive_closure``, C++ ``rb_matrix @``).  Inputs where the reference would never return
(its MSB loop on a negative signed operand) are detected first with the oracle and recorded
without a reference answer.  Output: ``tests/golden/golden.npz`` + ``tests/golden/index.json``.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import refimport, oracle as O  # noqa: E402
from redblackgraph_gb300 import synth  # noqa: E402

DTYPES = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64]


def exc_name(e):
    return type(e).__name__


_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from oracle import refimport
refimport.load()
import redblackgraph.core as core
from redblackgraph.core.redblack import array as rb_array
A = np.load(sys.argv[2])
try:
    W, d = core.warshall(np.stack([A, A]).view(rb_array))
    np.save(sys.argv[3], np.asarray(W[0]))
    print("OK", int(np.asarray(d).reshape(-1)[0]))
except Exception as e:
    print("EXC", type(e).__name__)
"""


def ref_warshall_isolated(A):
    """Run the reference gufunc in a child process: on an error it calls PyErr_Format from a
    loop NumPy may run with the GIL released, which can crash the interpreter."""
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "a.npy", Path(td) / "w.npy"
        np.save(fin, A)
        r = subprocess.run([sys.executable, "-c", _CHILD, str(ROOT), str(fin), str(fout)],
                           capture_output=True, text=True, timeout=120)
        out = r.stdout.strip().split()
        if r.returncode != 0 or not out:
            return "crash", None, None
        if out[0] == "OK":
            return "ok", np.load(fout), int(out[1])
        return out[1], None, None


_CHILD_COMPOSE = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from oracle import refimport
refimport.load()
import redblackgraph.core as core
from redblackgraph.core.redblack import array as rb_array
z = np.load(sys.argv[2])
try:
    if str(z["kind"]) == "vertex":
        out = core.vertex_relational_composition(z["u"], rb_array(z["R"]), z["v"], int(z["c"]))
    else:
        out = core.edge_relational_composition(rb_array(z["R"]), int(z["alpha"]), int(z["beta"]), int(z["rel"]))
    np.save(sys.argv[3], np.asarray(out))
    print("OK")
except Exception as e:
    print("EXC", type(e).__name__)
"""


def ref_compose_isolated(**kw):
    """The reference's C core composition in a child process (errors are raised from a gufunc
    loop, which can take the interpreter down)."""
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "a.npz", Path(td) / "w.npy"
        np.savez(fin, **kw)
        r = subprocess.run([sys.executable, "-c", _CHILD_COMPOSE, str(ROOT), str(fin), str(fout)],
                           capture_output=True, text=True, timeout=120)
        out = r.stdout.strip().split()
        if r.returncode != 0 or not out:
            return "crash", None
        if out[0] == "OK":
            return "ok", np.load(fout)
        return out[1], None


def compose_cases():
    """(name, kind, R, args) for relational composition: the reference's own test graphs, and
    closed pedigrees with a new vertex (parents u, children v) or a new edge."""
    cases = []
    A5 = np.array([[-1, 2, 3, 4, 0], [0, -1, 0, 2, 0], [0, 0, 1, 0, 0], [0, 0, 0, -1, 0], [2, 4, 5, 8, 1]])
    cases.append(("sibling", "vertex", A5, dict(u=np.array([2, 0, 0, 0, 0]), v=np.zeros(5, np.int64), c=-1)))
    R5 = np.array([[-1, 0, 3, 0, 0], [0, -1, 0, 2, 0], [0, 0, 1, 0, 0], [0, 0, 0, -1, 0], [2, 0, 5, 0, 1]])
    cases.append(("edge5", "edge", R5, dict(alpha=0, beta=1, rel=2)))
    cases.append(("edge5_zero_rel", "edge", R5, dict(alpha=0, beta=1, rel=0)))
    rng = np.random.default_rng(5)
    for n, g, seed in [(30, 5, 1), (60, 7, 2), (90, 9, 3)]:
        P = synth.pedigree(n, g, seed, dtype=np.int64)
        W, _, st, _ = O.warshall(P)
        assert st == 0
        anc = lambda x: set(np.nonzero(W[x])[0])  # noqa: E731
        for t in range(3):
            f, m = rng.choice(n, size=2, replace=False)
            u = np.zeros(n, np.int64)
            u[f], u[m] = 2, 3
            up = anc(f) | anc(m)
            kids = [k for k in rng.choice(n, size=4, replace=False) if k not in up and not (set(np.nonzero(W[:, k])[0]) & up)]
            v = np.zeros(n, np.int64)
            for k in kids[:2]:
                v[k] = 2 if k % 2 else 3
            cases.append((f"ped{n}_v{t}", "vertex", W, dict(u=u, v=v, c=-1 if t % 2 else 1)))
            # a cycle: a child that is also an ancestor of the parents
            if t == 0:
                vc = v.copy()
                vc[f] = 2
                cases.append((f"ped{n}_cycle", "vertex", W, dict(u=u, v=vc, c=1)))
        for t in range(3):
            while True:
                a, b = rng.choice(n, size=2, replace=False)
                if W[b, a] == 0 and W[a, b] == 0:
                    break
            cases.append((f"ped{n}_e{t}", "edge", W, dict(alpha=int(a), beta=int(b), rel=int(2 + t % 2))))
    # overflow: deep chains in narrow types
    for depth in (6, 8):
        nn = depth + 1
        C = np.zeros((nn, nn), np.int64)
        np.fill_diagonal(C, [(-1 if i % 2 == 0 else 1) for i in range(nn)])
        for i in range(nn - 1):
            C[i + 1, i] = 2 if i % 2 == 0 else 3
        W, _, st, _ = O.warshall(C)
        u = np.zeros(nn, np.int64)
        u[0] = 2
        cases.append((f"chain{depth}_v", "vertex", W, dict(u=u, v=np.eye(nn, dtype=np.int64)[nn - 1] * 3, c=1)))
        cases.append((f"chain{depth}_e", "edge", W, dict(alpha=nn - 1, beta=0, rel=2)))
    return cases


def main():
    rbg = refimport.load()
    import redblackgraph.core as core
    from redblackgraph.core.redblack import array as rb_array
    import redblackgraph.sparse.csgraph as csgraph
    from redblackgraph.sparse import rb_matrix

    arrays = {}
    index = {"scalar": {}, "warshall": [], "cython": [], "matmul": [], "spgemm": [], "dijkstra": []}

    # ---------------------------------------------------------------- scalar tables
    r = list(range(-1, 16))
    prod = np.array([[int(core.avos_product(x, y)) for y in r] for x in r], dtype=np.int64)
    arrays["scalar_product_table"] = prod
    r2 = list(range(-1, 4))
    arrays["scalar_sum_table"] = np.array([[int(core.avos_sum(x, y)) for y in r2] for x in r2], np.int64)
    index["scalar"]["edge_product"] = [str(9223372036854775807), "2", str(int(core.avos_product(9223372036854775807, 2)))]
    ovf = []
    for x, y in [(4294967296, 4294967296), (9223372036854775807, 3)]:
        try:
            core.avos_product(x, y)
            ovf.append([str(x), str(y), "none"])
        except Exception as e:  # noqa: BLE001
            ovf.append([str(x), str(y), exc_name(e)])
    index["scalar"]["overflow"] = ovf

    # ---------------------------------------------------------------- warshall inputs
    cases = []
    ex5 = np.array([[-1, 2, 3, 0, 0], [0, -1, 0, 2, 0], [0, 0, 1, 0, 0], [0, 0, 0, -1, 0],
                    [2, 0, 0, 0, 1]])
    for dt in DTYPES:
        cases.append(("example5", ex5.astype(dt)))
    for n, g, s in [(7, 3, 1), (33, 5, 2), (64, 6, 3), (65, 7, 4), (100, 8, 5), (130, 9, 6),
                    (200, 10, 7), (257, 12, 8), (300, 25, 9)]:
        for dt in (np.int32, np.int64, np.uint32, np.int16):
            cases.append((f"pedigree_n{n}_s{s}", synth.pedigree(n, g, s, dtype=dt)))
    # the reference's random-test style: triu(randint(0,4), 1) with a +-1 diagonal
    for seed in (42, 123, 456):
        rs = np.random.RandomState(seed)
        A = np.triu(rs.randint(0, 4, size=(20, 20)), k=1)
        np.fill_diagonal(A, rs.choice([-1, 1], size=20))
        for dt in (np.int32, np.int64):
            cases.append((f"randtriu_s{seed}", A.astype(dt)))
    # cycles
    cyc = synth.pedigree(40, 6, 11, dtype=np.int32)
    cyc[3, 30] = 2
    cases.append(("cycle40", cyc))
    cyc2 = synth.pedigree(150, 8, 12, dtype=np.int64)
    cyc2[5, 140] = 3
    cyc2[140, 5] = 2
    cases.append(("cycle150", cyc2))
    # deep chains: overflow / top-bit behaviour at small widths
    for dt, depth in [(np.uint8, 9), (np.uint16, 17), (np.int8, 6), (np.int16, 14),
                      (np.uint8, 7), (np.int32, 20)]:
        n = depth + 1
        A = np.zeros((n, n), np.int64)
        np.fill_diagonal(A, [(-1 if i % 2 == 0 else 1) for i in range(n)])
        for i in range(n - 1):
            A[i + 1, i] = 2 if i % 2 == 0 else 3
        cases.append((f"chain_{np.dtype(dt).name}_{depth}", A.astype(dt)))
    # small error cases the reference answers without crashing (< ~300 cells)
    c6 = np.zeros((6, 6), np.int64)
    np.fill_diagonal(c6, [-1, 1, -1, 1, -1, 1])
    c6[0, 1], c6[1, 2], c6[2, 3], c6[3, 0], c6[4, 0] = 3, 2, 3, 2, 2
    for dt in (np.int32, np.uint32, np.int64):
        cases.append(("cycle6", c6.astype(dt)))
    c12 = synth.pedigree(12, 4, 5, dtype=np.int64)
    c12[2, 11] = 2
    cases.append(("cycle12", c12.astype(np.int32)))
    for dt, depth in [(np.uint8, 8), (np.uint8, 10), (np.uint16, 16), (np.int8, 7), (np.int8, 8),
                      (np.int16, 15), (np.uint32, 15)]:
        n = depth + 1
        A = np.zeros((n, n), np.int64)
        np.fill_diagonal(A, [(-1 if i % 2 == 0 else 1) for i in range(n)])
        for i in range(n - 1):
            A[i + 1, i] = 3 if i % 2 == 0 else 2
        if dt == np.uint32:   # wide edges: every edge spans 3 generations (values 8..15)
            for i in range(n - 1):
                A[i + 1, i] = 8 + (i % 8)
        cases.append((f"chain3_{np.dtype(dt).name}_{depth}", A.astype(dt)))
    # overflow and a cycle in one matrix: the reference raises the LAST error it set
    oc = np.zeros((10, 10), np.int64)
    np.fill_diagonal(oc, 1)
    for i in range(9):
        oc[i + 1, i] = 3
    oc[0, 9] = 3
    for dt in (np.uint8, np.int8, np.uint16):
        cases.append(("ovf_cycle10", oc.astype(dt)))
    # first-found longer than final (diameter counts values later replaced)
    A = np.zeros((5, 5), np.int32)
    np.fill_diagonal(A, [-1, -1, 1, -1, 1])
    A[0, 1], A[1, 2], A[2, 3], A[0, 4], A[4, 3] = 2, 3, 2, 3, 2
    cases.append(("first_found", A))

    for ci, (name, A) in enumerate(cases):
        key = f"w{ci}"
        arrays[key + "_in"] = A
        Wo, do, so, info = O.warshall(A)
        rec = {"key": key, "name": name, "dtype": np.dtype(A.dtype).name, "n": int(A.shape[0])}
        if info[1] & O.EV_HANG:
            rec["reference"] = "hang"
            rec["exception"] = "OverflowError"
        elif so != 0:
            kind, W2, d2 = ref_warshall_isolated(A)
            if kind == "crash":
                rec["reference"] = "crash"
                rec["exception"] = {1: "OverflowError", 2: "ValueError"}[so]
            elif kind == "ok":
                arrays[key + "_W"] = W2
                rec["diameter"] = d2
                rec["exception"] = None
            else:
                rec["exception"] = kind
        else:
            try:
                # The reference gufunc stores its diameter as an 8-byte npy_intp into a 4-byte
                # int32 slot (warshall.c.in:106,146-149) and never advances that pointer over a
                # batch (:128).  Closing a 2-stack of the same matrix keeps the spill in bounds.
                W2, d2 = core.warshall(np.stack([A, A]).view(rb_array))
                arrays[key + "_W"] = np.asarray(W2[0])
                rec["diameter"] = int(np.asarray(d2).reshape(-1)[0])
                rec["exception"] = None
            except Exception as e:  # noqa: BLE001
                rec["exception"] = exc_name(e)
        index["warshall"].append(rec)

        # Cython floyd_warshall on the int32 view (what validate_graph makes)
        if A.dtype == np.int32:
            for tri in ((False, True) if not np.tril(A, -1).any() else (False,)):
                rec2 = {"key": key, "name": name, "triangular": tri}
                try:
                    W2, d2 = csgraph.floyd_warshall(A.copy(), assume_upper_triangular=tri)
                    arrays[key + ("_cyT" if tri else "_cy")] = np.asarray(W2)
                    rec2["diameter"] = int(d2)
                    rec2["exception"] = None
                except Exception as e:  # noqa: BLE001
                    rec2["exception"] = exc_name(e)
                    rec2["vertex"] = int(getattr(e, "vertex", -1))
                index["cython"].append(rec2)

    # ---------------------------------------------------------------- dense @
    mm = [("example5", ex5)]
    for s in (1, 2):
        mm.append((f"ped40_s{s}", synth.pedigree(40, 6, s, dtype=np.int64)))
    for ci, (name, A) in enumerate(mm):
        for dt in DTYPES:
            a = A.astype(dt)
            key = f"m{ci}_{np.dtype(dt).name}"
            arrays[key + "_in"] = a
            rec = {"key": key, "name": name}
            try:
                C = rb_array(a) @ rb_array(a)
                arrays[key + "_AA"] = np.asarray(C)
                rec["exception"] = None
            except Exception as e:  # noqa: BLE001
                rec["exception"] = exc_name(e)
            index["matmul"].append(rec)

    # ---------------------------------------------------------------- rb_matrix @ (C++)
    for ci, (n, g, s, dt) in enumerate([(50, 6, 1, np.int32), (200, 10, 2, np.int64),
                                        (300, 12, 3, np.int32), (120, 8, 4, np.uint32)]):
        M = synth.pedigree_csr(n, g, s, dtype=dt)
        key = f"s{ci}"
        arrays[key + "_indptr"], arrays[key + "_indices"], arrays[key + "_data"] = M.indptr, M.indices, M.data
        R = rb_matrix(M)
        C = (R @ R).tocsr()
        C2 = sp.csr_matrix(C)
        C2.sort_indices()
        arrays[key + "_C_indptr"], arrays[key + "_C_indices"], arrays[key + "_C_data"] = C2.indptr, C2.indices, C2.data
        index["spgemm"].append({"key": key, "n": n, "dtype": np.dtype(dt).name})

    # ---------------------------------------------------------------- csgraph 'D' closure
    for ci, (n, g, s) in enumerate([(60, 6, 21), (150, 9, 22)]):
        M = synth.pedigree_csr(n, g, s, dtype=np.int32)
        key = f"d{ci}"
        arrays[key + "_in"] = M.toarray()
        res = csgraph.transitive_closure(M, method="D")
        arrays[key + "_W"] = np.asarray(res.W)
        index["dijkstra"].append({"key": key, "diameter": int(res.diameter)})

    # ---------------------------------------------------------------- component-wise closure
    index["components"] = []
    for ci, (sizes, seed, method, thr, cyc) in enumerate([
            ([30, 5, 80, 1, 45, 12], 31, "auto", 40, False),
            ([30, 5, 80, 1, 45, 12], 31, "FW", 500, False),
            ([30, 5, 80, 1, 45, 12], 31, "D", 500, False),
            ([70], 32, "auto", 500, False),
            ([70], 32, "FW", 500, False),
            ([20, 35, 9], 33, "auto", 500, True)]):
        blocks = [synth.pedigree_csr(n, max(2, n // 8), seed + j, dtype=np.int32)
                  for j, n in enumerate(sizes)]
        M = sp.block_diag(blocks, format="csr").astype(np.int32)
        perm = np.random.default_rng(seed).permutation(M.shape[0])
        M = sp.csr_matrix(M[perm][:, perm])
        if cyc:                                   # a cycle inside the second component
            M = M.tolil()
            rows = np.flatnonzero(np.isin(perm, np.arange(20, 55)))
            Mc = M[rows][:, rows].tocoo()
            off = Mc.row != Mc.col
            a, b = rows[Mc.row[off][0]], rows[Mc.col[off][0]]
            M[b, a] = 2
            M = M.tocsr()
        M.sort_indices()
        key = f"c{ci}"
        arrays[key + "_indptr"], arrays[key + "_indices"], arrays[key + "_data"] = M.indptr, M.indices, M.data
        rec = {"key": key, "n": int(M.shape[0]), "method": method, "threshold": thr}
        try:
            res = csgraph.component_wise_closure(M, method=method, densify_threshold=thr)
            W = sp.csr_matrix(res.W)
            W.sort_indices()
            arrays[key + "_W_indptr"], arrays[key + "_W_indices"], arrays[key + "_W_data"] = W.indptr, W.indices, W.data
            rec["diameter"] = int(res.diameter)
        except Exception as e:
            rec["error"] = exc_name(e)
            rec["vertex"] = getattr(e, "vertex", None)
        index["components"].append(rec)

    # ---------------------------------------------------------------- relationship lookups
    from redblackgraph.reference import calculate_relationship
    index["relationship"] = []
    for ci, (n, g, sd, dt) in enumerate([(120, 8, 41, np.int32), (90, 7, 42, np.uint32),
                                         (200, 10, 43, np.int64)]):
        A = synth.pedigree(n, g, sd, dtype=np.int64)
        W, _, st, _ = O.warshall(A)
        assert st == 0
        W = W.astype(dt)                      # the red one -1 becomes the unsigned maximum
        key = f"r{ci}"
        arrays[key + "_W"] = W
        rng = np.random.default_rng(sd)
        pairs = rng.integers(0, n, size=(150, 2))
        out = []
        for u, v in pairs:
            with np.errstate(over="ignore"):
                rel = calculate_relationship(list(W[u]), list(W[v]))
            out.append([int(u), int(v), int(rel.common_ancestor), rel.relationship])
        index["relationship"].append({"key": key, "pairs": out})

    # ---------------------------------------------------------------- sparse DAG closure
    index["dag"] = []
    for ci, seed in enumerate([0, 1, 2, 6]):
        M = sp.csr_matrix(synth.forest(600, 12, seed, family=60, reach=3, dtype=np.int32))
        M.sort_indices()
        key = f"g{ci}"
        arrays[key + "_indptr"], arrays[key + "_indices"], arrays[key + "_data"] = M.indptr, M.indices, M.data
        res = csgraph.transitive_closure_dag_sparse(M)
        W = sp.csr_matrix(res.W)
        W.sort_indices()
        arrays[key + "_W_indptr"], arrays[key + "_W_indices"], arrays[key + "_W_data"] = W.indptr, W.indices, W.data
        mxf = int(np.abs(W.data).max())
        index["dag"].append({"key": key, "n": int(M.shape[0]), "diameter": int(res.diameter),
                             "final_max_msb": (mxf.bit_length() - 1) if mxf > 1 else 0})

    # ---------------------------------------------------------------- adaptive dispatch, components
    index["adaptive"] = []
    perm_tri = synth.pedigree_csr(120, 8, 71)
    p = np.random.default_rng(71).permutation(120)
    cases = [("forest", sp.csr_matrix(sp.block_diag([synth.pedigree_csr(n, 5, 72 + j) for j, n in
                                                         enumerate([30, 12, 50])]).astype(np.int32)), {}),
             ("tri", sp.csr_matrix(synth.pedigree_csr(150, 9, 73)), {}),
             ("perm", sp.csr_matrix(perm_tri[p][:, p]), {}),
             ("perm_dag", sp.csr_matrix(perm_tri[p][:, p]), {"method": "dag_sparse"}),
             ("sparse_only_cycle", sp.csr_matrix(np.array([[-1, 2, 0], [0, 1, 3], [2, 0, -1]], dtype=np.int32)),
              {"sparse_only": True})]
    for ci, (name, M, kw) in enumerate(cases):
        key = f"ad{ci}"
        M.sort_indices()
        arrays[key + "_indptr"], arrays[key + "_indices"], arrays[key + "_data"] = M.indptr, M.indices, M.data
        rec = {"key": key, "name": name, "n": int(M.shape[0]), "kwargs": kw}
        q = {}
        arrays[key + "_labels"] = np.asarray(csgraph.find_components_sparse(M, q)).astype(np.int64)
        rec["q"] = {str(k): int(v) for k, v in q.items()}
        try:
            res = csgraph.transitive_closure_adaptive(M, **kw)
            W = sp.csr_matrix(res.W)
            W.sort_indices()
            arrays[key + "_W_indptr"], arrays[key + "_W_indices"], arrays[key + "_W_data"] = W.indptr, W.indices, W.data
            rec["diameter"] = int(res.diameter)
        except Exception as e:
            rec["error"] = exc_name(e)
        index["adaptive"].append(rec)

    # ---------------------------------------------------------------- relational composition
    index["compose"] = []
    ci = 0
    for name, kind, R, args in compose_cases():
        for dt in ([np.int32] if name.startswith("ped9") else DTYPES):
            if kind == "edge" and np.iinfo(dt).max < R.shape[0]:
                continue
            Rt = R.astype(dt)
            key = f"rc{ci}"
            ci += 1
            arrays[key + "_R"] = Rt
            rec = {"key": key, "name": name, "kind": kind, "dtype": np.dtype(dt).name}
            if kind == "vertex":
                u, v = args["u"].astype(dt), args["v"].astype(dt)
                arrays[key + "_u"], arrays[key + "_v"] = u, v
                rec["c"] = int(args["c"])
                _, info = O.vertex_compose(Rt, u, v, rec["c"])
                kw = dict(kind="vertex", R=Rt, u=u, v=v, c=rec["c"])
            else:
                rec.update(alpha=args["alpha"], beta=args["beta"], rel=args["rel"])
                _, info = O.edge_compose(Rt, args["alpha"], args["beta"], args["rel"])
                kw = dict(kind="edge", R=Rt, alpha=args["alpha"], beta=args["beta"], rel=args["rel"])
            if info[0] and (info[7] & O.EV_HANG):
                rec["hang"] = True               # the reference would not return
            else:
                st, out = ref_compose_isolated(**kw)
                if st == "ok":
                    arrays[key + "_out"] = out.astype(dt)
                else:
                    rec["error"] = st
            # the Cython functions (int32 only, no cycle check, silent wrap)
            if dt == np.int32 and R.shape[0] < 100:
                try:
                    if kind == "vertex":
                        cy = csgraph.vertex_relational_composition(u.copy(), Rt.copy(), v.copy(), rec["c"])
                    else:
                        cy = csgraph.edge_relational_composition(Rt.copy(), args["alpha"], args["beta"], args["rel"])
                    arrays[key + "_cy"] = np.asarray(cy)
                except Exception as e:  # noqa: BLE001
                    rec["cy_error"] = exc_name(e)
            index["compose"].append(rec)

    # ---------------------------------------------------------------- orderings
    index["ordering"] = []
    import scipy.sparse as sp2
    rng2 = np.random.default_rng(17)
    for oi, (sizes, seed) in enumerate([((20, 35, 12, 35, 1, 1), 3), ((60, 60, 9), 4), ((150,), 5),
                                        ((7, 7, 7, 3, 3, 40), 6)]):
        blocks = []
        for j, m in enumerate(sizes):
            P = synth.pedigree(m, max(2, int(np.log2(m + 1)) + 1), seed * 31 + j, dtype=np.int64)
            W, _, st, _ = O.warshall(P)
            blocks.append(W)
        from scipy.linalg import block_diag
        M = block_diag(*blocks).astype(np.int32)
        p = rng2.permutation(M.shape[0])
        M = np.ascontiguousarray(M[p][:, p])             # interleave the components
        key = f"ord{oi}"
        arrays[key + "_A"] = M
        dense = csgraph.avos_canonical_ordering(rb_array(M))
        arrays[key + "_perm_dense"] = np.asarray(dense.label_permutation, np.int32)
        arrays[key + "_B_dense"] = np.asarray(dense.A)
        S = sp2.csr_matrix(M)
        sparse = csgraph.avos_canonical_ordering(S)
        arrays[key + "_perm_sparse"] = np.asarray(sparse.label_permutation, np.int32)
        Bs = sp2.csr_matrix(sparse.A)
        arrays[key + "_B_indptr"], arrays[key + "_B_indices"], arrays[key + "_B_data"] = Bs.indptr, Bs.indices, Bs.data
        rp = rng2.permutation(M.shape[0]).astype(np.int32)
        arrays[key + "_rp"] = rp
        arrays[key + "_permute_full"] = np.asarray(csgraph.permute(M, rp))
        arrays[key + "_permute_upper"] = np.asarray(csgraph.permute(M, rp, assume_upper_triangular=True))
        Pu = sp2.csr_matrix(csgraph.permute_sparse(S, rp, assume_upper_triangular=True))
        arrays[key + "_ps_indptr"], arrays[key + "_ps_indices"], arrays[key + "_ps_data"] = Pu.indptr, Pu.indices, Pu.data
        arrays[key + "_topo"] = np.asarray(csgraph.topological_sort(S), np.int32)
        # extract every component, then merge them back
        q2 = {}
        lab = csgraph.find_components_sparse(S, q2)
        parts = []
        for c, verts in sorted(csgraph.get_component_vertices(lab).items()):
            sub, mp = csgraph.extract_submatrix(S, verts)
            sub = sp2.csr_matrix(sub)
            arrays[f"{key}_sub{c}_indptr"], arrays[f"{key}_sub{c}_indices"], arrays[f"{key}_sub{c}_data"] = (
                sub.indptr, sub.indices, sub.data)
            arrays[f"{key}_sub{c}_map"] = np.asarray(mp, np.int32)
            parts.append((sub, mp))
        Mg = sp2.csr_matrix(csgraph.merge_component_matrices(parts, M.shape[0]))
        arrays[key + "_merged_indptr"], arrays[key + "_merged_indices"], arrays[key + "_merged_data"] = (
            Mg.indptr, Mg.indices, Mg.data)
        index["ordering"].append({"key": key, "n": int(M.shape[0]), "ncomp": len(parts),
                                  "q_dense": {str(k): int(v) for k, v in dense.components.items()},
                                  "q_sparse": {str(k): int(v) for k, v in sparse.components.items()}})

    np.savez_compressed(HERE / "golden.npz", **arrays)
    (HERE / "index.json").write_text(json.dumps(index, indent=1))
    print(f"wrote {len(arrays)} arrays, {len(index['warshall'])} warshall cases")


if __name__ == "__main__":
    main()
