"""The multi-rank bench path on CPU: two gloo ranks, each transforming its own
batch (no data-path collective), the step time reduced with MAX over ranks and
the per-rank results gathered on rank 0 to check the split against a single
process.  The transforms run in the oracle's CPU port, standing in for one
GPU per rank (this container has none)."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import torch
    from oracle import oracle as O
    dist.init_process_group("gloo")
    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    n, batch = 256, 6
    rng = np.random.default_rng(bench.rank_seed(r))
    a = rng.standard_normal(n * batch).astype(np.float32)
    b = rng.standard_normal(n * batch).astype(np.float32)
    yr, yi = O.Port32("c", [n])(a, b, batch=batch)
    t = torch.tensor([0.5 + rank])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)     # the bench's max-over-ranks timing
    gathered = [None] * world
    dist.all_gather_object(gathered, (r, a, b, yr, yi, float(t.item())))
    if r == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from oracle import oracle as O
    assert [g[0] for g in got] == [0, 1]
    assert all(g[5] == 1.5 for g in got)   # MAX over ranks
    # each rank's inputs differ (own seed); each rank's outputs match a
    # single-process transform of the same inputs
    assert not np.array_equal(got[0][1], got[1][1])
    for _, a, b, yr, yi, _ in got:
        ref = O.Port32("c", [256])(a, b, batch=6)
        assert np.array_equal(ref[0], yr) and np.array_equal(ref[1], yi)
