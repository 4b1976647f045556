"""Full-size parity fixtures made by running the reference itself on the bench's own inputs.

Run in a container where the reference tree is mounted and built (``python oracle/ref_build.py``):

    python tests/golden/make_fullsize.py dense8192     # ~45 min: C core warshall, n=8192, int64
    python tests/golden/make_fullsize.py forest2m      # ~1 min: Cython DAG closure, 2,000,000 vertices
    python tests/golden/make_fullsize.py served4111    # ~5 min: C core warshall, n=4111, int64

Each case closes one of the bench's seeded inputs with the reference's own CPU code and stores
digests, not matrices (a closed n=8192 int64 matrix is 512 MiB): the SHA-256 of the input (so a
change of the generator shows up as a stale fixture, not as a parity failure), the SHA-256 of the
closure, its diameter, the exception the reference raised (or none) and the number of non-zeros.
Output: ``tests/golden/fullsize.json`` (one entry per case, merged into the file).

* ``dense8192``  -- ``synth.pedigree(8192, 30, seed=1)`` in int64, the single dense closure of the
  bench, through the C core ``warshall`` gufunc (``core/src/redblackgraph/warshall.c.in:51-107``).
* ``forest2m``   -- ``synth.forest(2_000_000, 25, seed=7, family=64, reach=3, p_parent=0.97)`` in
  int32, the bench's squaring and DAG-closure forest, through the Cython
  ``transitive_closure_dag_sparse`` (``sparse/csgraph/_transitive_closure_dag.pyx:168-351``); its
  closure is the fixed point of the squaring loop as well.
* ``served4111`` -- the smallest int64 graph of the bench's serving stream (request 2027:
  ``pedigree_csr(4111, generations_for(4111), seed=608998870)``), through the C core ``warshall``.

The reference's gufunc writes its diameter as an 8-byte integer into an int32 slot
(``warshall.c.in:106,146-149``); the single-matrix call therefore gets a 0-d output that views
the first element of a larger int32 buffer.  Each case runs in a child process, because the
gufunc sets Python errors from a loop that can run without the GIL.
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "fullsize.json"

CASES = {
    "dense8192": dict(kind="dense", n=8192, generations=30, seed=1, dtype="int64"),
    "forest2m": dict(kind="forest", n=2_000_000, generations=25, seed=7, family=64, reach=3,
                     p_parent=0.97, dtype="int32"),
    "served4111": dict(kind="served", n=4111, seed=608998870, dtype="int64"),
}


def dense_digest(W) -> str:
    """SHA-256 of a dense matrix's bytes, row-major, in its own storage type."""
    return hashlib.sha256(np.ascontiguousarray(W).tobytes()).hexdigest()


def csr_digest(M) -> str:
    """SHA-256 of a sparse matrix in a canonical form: CSR without stored zeros, columns
    ascending, row pointers as int64, columns as int32, values as int64."""
    import scipy.sparse as sp
    M = sp.csr_matrix(M, copy=True)
    M.sum_duplicates()
    M.eliminate_zeros()
    M.sort_indices()
    h = hashlib.sha256()
    h.update(np.asarray(M.indptr, dtype=np.int64).tobytes())
    h.update(np.asarray(M.indices, dtype=np.int32).tobytes())
    h.update(np.asarray(M.data, dtype=np.int64).tobytes())
    return h.hexdigest()


def make_input(name: str):
    """The case's input exactly as the bench builds it (dense array or scipy CSR)."""
    sys.path.insert(0, str(ROOT))
    from redblackgraph_gb300 import synth
    c = CASES[name]
    if c["kind"] == "dense":
        return synth.pedigree(c["n"], c["generations"], c["seed"], dtype=np.dtype(c["dtype"]))
    if c["kind"] == "forest":
        return synth.forest(c["n"], c["generations"], c["seed"], family=c["family"], reach=c["reach"],
                            p_parent=c["p_parent"], dtype=np.dtype(c["dtype"]))
    m = synth.pedigree_csr(c["n"], synth.generations_for(c["n"]), c["seed"])
    return m.toarray().astype(np.dtype(c["dtype"]))


def input_digest(name: str, A) -> str:
    return csr_digest(A) if CASES[name]["kind"] == "forest" else dense_digest(A)


_CHILD = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, sys.argv[1])
from oracle import refimport
refimport.load()
sys.path.insert(0, sys.argv[3])
from make_fullsize import CASES, make_input, input_digest, dense_digest, csr_digest
name = sys.argv[2]
A = make_input(name)
rec = {"input_sha256": input_digest(name, A)}
t0 = time.perf_counter()
try:
    if CASES[name]["kind"] == "forest":
        import redblackgraph.sparse.csgraph as csgraph
        import scipy.sparse as sp
        M = sp.csr_matrix(A)
        M.sort_indices()
        res = csgraph.transitive_closure_dag_sparse(M)
        W = sp.csr_matrix(res.W)
        rec.update(closure_sha256=csr_digest(W), diameter=int(res.diameter), nnz=int(sp.csr_matrix(W).count_nonzero()),
                   exception=None, reference_call="redblackgraph.sparse.csgraph.transitive_closure_dag_sparse")
    else:
        import redblackgraph.core as core
        from redblackgraph.core.redblack import array as rb_array
        slot = np.zeros(4, np.int32)
        d = slot[:1].reshape(())
        W = np.empty_like(A)
        core.warshall(A.view(rb_array), out=(W.view(rb_array), d))
        rec.update(closure_sha256=dense_digest(W), diameter=int(slot[0]), nnz=int(np.count_nonzero(W)),
                   exception=None, reference_call="redblackgraph.core.warshall")
except Exception as e:
    rec.update(exception=type(e).__name__)
rec["reference_seconds"] = round(time.perf_counter() - t0, 1)
print("RESULT " + json.dumps(rec))
"""


def run_case(name: str) -> dict:
    r = subprocess.run([sys.executable, "-c", _CHILD, str(ROOT), name, str(HERE)], capture_output=True, text=True)
    for line in r.stdout.splitlines():
        if line.startswith("RESULT "):
            rec = json.loads(line[7:])
            rec["case"] = dict(CASES[name])
            return rec
    raise RuntimeError(f"{name}: the reference run gave no result (rc {r.returncode})\n{r.stdout}\n{r.stderr}")


def main(argv):
    names = argv or list(CASES)
    for name in names:
        t0 = time.perf_counter()
        rec = run_case(name)
        # merge under a re-read, so that cases run in parallel processes keep each other's entries
        data = json.loads(OUT.read_text()) if OUT.exists() else {}
        data[name] = rec
        OUT.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
        print(f"{name}: diameter {rec.get('diameter')} exception {rec.get('exception')} "
              f"({time.perf_counter() - t0:.0f} s)")


if __name__ == "__main__":
    main(sys.argv[1:])
