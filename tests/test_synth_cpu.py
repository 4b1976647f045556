"""The synthetic pedigrees the bench and tests use: numbered oldest first (every parent edge
below the diagonal, the property the DAG path of the batched closure relies on) and in the
clean regime (diagonal -1/1, edge values 2 and 3), deterministic per seed."""
import numpy as np

from redblackgraph_gb300 import synth


def test_pedigrees_are_numbered_oldest_first_and_clean():
    for n, seed in ((16, 1), (300, 2), (2048, 3)):
        A = synth.pedigree(n, synth.generations_for(n), seed, dtype=np.int64)
        off = A - np.diag(np.diag(A))
        assert not np.triu(off).any()                     # parents have lower numbers
        assert set(np.unique(np.diag(A))) <= {-1, 1}
        assert set(np.unique(off[off != 0])) <= {2, 3}
        assert ((off != 0).sum(axis=1) <= 2).all()        # at most a father and a mother
        assert (synth.pedigree(n, synth.generations_for(n), seed, dtype=np.int64) == A).all()
        B = synth.pedigree_csr(n, synth.generations_for(n), seed, dtype=np.int64)
        assert (B.toarray() == A).all()


def test_batch_forest_blocks_keep_the_order():
    sizes, seeds = synth.batch_components(12, 4, 300, seed=5)
    F, _ = synth.batch_forest(sizes, seeds)
    F = F.tocoo()
    off = F.row != F.col
    assert (F.col[off] < F.row[off]).all()                # every component numbered oldest first
