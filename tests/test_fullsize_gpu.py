"""Full-size parity against the reference itself.

The fixtures in tests/golden/fullsize.json were made by tests/golden/make_fullsize.py, which
runs the reference's own CPU code (C core ``warshall``, Cython ``transitive_closure_dag_sparse``)
on the bench's seeded inputs and keeps SHA-256 digests of the inputs and closures with the
diameters.  Each test rebuilds the same input, checks its digest (a changed generator is a stale
fixture, not a parity failure), closes it on the GPU through the public entry points and
compares digests and diameters: bit-exact at the sizes the bench measures.
"""
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = json.loads((GOLDEN / "fullsize.json").read_text())


def _maker():
    spec = importlib.util.spec_from_file_location("make_fullsize", GOLDEN / "make_fullsize.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _case(name):
    if name not in FIXTURES:
        pytest.fail(f"fixture {name} missing from tests/golden/fullsize.json")
    mk = _maker()
    fx = FIXTURES[name]
    A = mk.make_input(name)
    assert mk.input_digest(name, A) == fx["input_sha256"], "input generator changed: remake the fixture"
    assert fx["exception"] is None
    return mk, fx, A


def test_dense_n8192_int64_matches_reference(native):
    """One pedigree of 8192 vertices in 30 generations, int64: the single dense closure of the
    bench, on the DAG path and on the blocked kernels, against the reference's warshall."""
    import torch
    import redblackgraph_gb300 as rbg
    from redblackgraph_gb300 import _lib
    from redblackgraph_gb300.dense import fw_dense
    from redblackgraph_gb300.device import to_device, to_host
    mk, fx, A = _case("dense8192")
    res = rbg.array(A).transitive_closure()              # the drop-in for rb.array.transitive_closure
    W = np.asarray(res.W)
    assert mk.dense_digest(W) == fx["closure_sha256"]
    assert int(res.diameter) == fx["diameter"]
    del W, res
    d = to_device(A)
    out, r = fw_dense(d, mode=_lib.MODE_NO_DAG)
    torch.cuda.synchronize()
    assert r.path in (_lib.PATH_BLOCKED32, _lib.PATH_BLOCKED64)
    assert mk.dense_digest(to_host(out)) == fx["closure_sha256"] and r.diameter == fx["diameter"]


def test_served_n4111_int64_matches_reference(native):
    """The smallest int64 graph of the bench's serving stream (request 2027 of the default run),
    served in a mix with int32 graphs and lookups on it: the resident closure and its diameter
    against the reference's warshall."""
    from redblackgraph_gb300.serving import GpuExecutor, Policy, Request, Server, make_stream
    mk, fx, A = _case("served4111")
    case = fx["case"]
    mix = make_stream(24, 4000.0, 0.3, 64, 3000, seed=31)
    big = len(mix)
    reqs = mix + [Request(big, "closure", mix[-1].arrival, n=case["n"], seed=case["seed"])]
    reqs += [Request(big + 1 + k, "lookup", mix[-1].arrival + 1e-4, target=big, u=k, v=case["n"] - 1 - k)
             for k in range(3)]
    cap = 2 << 30
    ex = GpuExecutor(arena_bytes=cap, slots=2, keep=True)
    ex.prepare(reqs)
    Server(ex, cap, Policy(inflight=2, max_batch=64)).run(reqs)
    W = ex.kept[big]
    assert W.dtype == np.int64
    assert mk.dense_digest(W) == fx["closure_sha256"]
    assert reqs[big].result == (0, fx["diameter"])
    ex.close()


def test_forest_2m_closures_match_reference(native):
    """The bench's 2,000,000-vertex forest (25 generations): the closure by levels (the drop-in
    transitive_closure_dag_sparse) and the fixed point of the squaring SpGEMM loop, against the
    reference's Cython DAG closure."""
    import torch
    from redblackgraph_gb300.sparse import transitive_closure_dag_sparse
    from redblackgraph_gb300.spgemm import DeviceCSR, SEM_C64, spgemm
    mk, fx, A = _case("forest2m")
    r = transitive_closure_dag_sparse(A)
    assert mk.csr_digest(r.W) == fx["closure_sha256"]
    assert int(r.diameter) == fx["diameter"]
    R = DeviceCSR.from_scipy(A, dtype=np.int64)
    for _ in range(64):
        Rn, rc, _ = spgemm(R, R, R=R, sem=SEM_C64)
        assert rc == 0
        if Rn.equal(R):
            break
        R = Rn
    torch.cuda.synchronize()
    assert mk.csr_digest(Rn.to_scipy()) == fx["closure_sha256"]
