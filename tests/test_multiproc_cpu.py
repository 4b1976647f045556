"""The multi-GPU host logic with two gloo ranks on the CPU: every rank computes the same split of
a batch (a partition of the components, balanced by n^3), closes its share with the oracle, and
the slowest rank's time is what every rank reports.  No GPU is used."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sharding import max_over_ranks, shard_components
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes, seeds = synth.batch_components(40, 4, 120, seed=3)
        parts = shard_components(sizes, world)
        mine = parts[rank]
        closed = {}
        for i in mine:                                   # this rank's share, closed alone
            A = synth.pedigree(int(sizes[i]), synth.generations_for(int(sizes[i])), int(seeds[i]))
            W, d, st, _ = O.warshall(A)
            closed[int(i)] = (int(d), int(st), int((W != 0).sum()))
        slowest = max_over_ranks(0.5 + rank)             # each rank's "time"
        q.put((rank, [p.tolist() for p in parts], closed, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_and_reduce():
    import torch.multiprocessing as mp
    from redblackgraph_gb300 import synth
    from redblackgraph_gb300.sharding import shard_components, shard_cost
    from oracle import oracle as O
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    splits = [o[1] for o in out]
    assert splits[0] == splits[1]                        # both ranks agree on the split
    sizes, seeds = synth.batch_components(40, 4, 120, seed=3)
    allidx = sorted(i for part in splits[0] for i in part)
    assert allidx == list(range(len(sizes)))             # a partition: every component once
    costs = shard_cost(sizes, [np.array(p) for p in splits[0]])
    assert costs.max() <= 1.5 * costs.min() + float(sizes.max()) ** 3
    assert all(o[3] == 1.5 for o in out)                 # every rank reports the slowest time
    merged = {**out[0][2], **out[1][2]}
    for i in range(len(sizes)):                          # the union equals closing everything here
        A = synth.pedigree(int(sizes[i]), synth.generations_for(int(sizes[i])), int(seeds[i]))
        W, d, st, _ = O.warshall(A)
        assert merged[i] == (int(d), int(st), int((W != 0).sum()))


def test_split_is_deterministic_and_balanced():
    from redblackgraph_gb300.sharding import shard_components, shard_cost
    rng = np.random.default_rng(1)
    sizes = rng.integers(16, 4096, size=500)
    for world in (1, 2, 4, 8):
        parts = shard_components(sizes, world)
        assert [p.tolist() for p in parts] == [p.tolist() for p in shard_components(sizes, world)]
        assert sorted(np.concatenate(parts).tolist()) == list(range(500))
        c = shard_cost(sizes, parts)
        assert c.max() - c.min() <= float(sizes.max()) ** 3
    with pytest.raises(ValueError):
        shard_components(sizes, 0)
