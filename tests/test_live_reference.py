"""Oracle vs the reference itself on fresh seeded inputs (only where the reference is mounted
and built, i.e. not on the GPU host)."""
import numpy as np
import pytest

from oracle import oracle as O, refimport

pytestmark = pytest.mark.skipif(not refimport.available(), reason="reference not available here")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_warshall_matches_reference(seed):
    rbg = refimport.load()
    import redblackgraph.core as core
    from redblackgraph.core.redblack import array as rb_array
    from redblackgraph_gb300 import synth
    for n, g, dt in [(90, 8, np.int32), (140, 11, np.int64), (70, 30, np.int64)]:
        A = synth.pedigree(n, g, seed + n, dtype=dt)
        W, d = core.warshall(np.stack([A, A]).view(rb_array))
        Wo, do, so, _ = O.warshall(A)
        assert so == 0 and (Wo == np.asarray(W[0])).all() and do == int(np.asarray(d).reshape(-1)[0])


def test_cython_random_triu_matches_reference():
    rbg = refimport.load()
    import redblackgraph.sparse.csgraph as csgraph
    for seed in range(5):
        rs = np.random.RandomState(seed)
        A = np.triu(rs.randint(0, 4, size=(30, 30)), k=1)
        np.fill_diagonal(A, rs.choice([-1, 1], size=30))
        A = A.astype(np.int32)
        W, d = csgraph.floyd_warshall(A.copy())
        Wo, do, so, _ = O.fw_cython(A)
        assert so == 0 and (Wo == np.asarray(W)).all() and do == d
