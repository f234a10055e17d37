"""Host logic of the N > 1 bench paths on CPU ranks (gloo, world size 2):
the batched problems are sharded with no data-path collective and every
rank computes the same partition; the job's time is the slowest rank's and
its counts are summed over ranks.  No GPU is involved."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = bench.shard_problems(costs, rank, world)
        load = sum(costs[i] for i in mine)
        mx = bench.reduce_ranks([10.0 + rank, -rank], "max", world)
        sm = bench.reduce_ranks([len(mine), load], "sum", world)
        out.put((rank, mine, load, mx, sm))
    finally:
        dist.destroy_process_group()


def test_batched_sharding_and_reductions_on_two_gloo_ranks():
    import numpy as np
    import torch.multiprocessing as mp
    rng = np.random.default_rng(1)
    costs = [int(c) for c in rng.integers(1_000, 2_000_000, 61)]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, costs, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shards = [set(r[1]) for r in res]
    assert shards[0].isdisjoint(shards[1]) and shards[0] | shards[1] == set(range(len(costs)))
    loads = [r[2] for r in res]
    assert abs(loads[0] - loads[1]) <= max(costs)  # LPT balance
    for r in res:
        assert r[3] == [11.0, 0.0]  # max over ranks
        assert r[4] == [float(len(costs)), float(sum(costs))]  # sums over ranks


def test_single_rank_reductions_are_identity():
    import bench
    assert bench.reduce_ranks([3, 4.5], "max", 1) == [3.0, 4.5]
    assert bench.shard_problems([5, 1, 3], 0, 1) == [0, 1, 2]
