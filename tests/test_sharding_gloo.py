"""Multi-process source sharding and max-over-ranks timing (gloo, CPU, world size 2)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from eikonalxx_gb300 import sharding  # noqa: E402


def test_shard_covers_every_item_once():
    for n in (0, 1, 5, 32, 33):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in range(n)[sharding.shard(n, world, r)]]
            assert got == list(range(n))
            sizes = [len(range(n)[sharding.shard(n, world, r)]) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sharding.shard(4, 2, 2)


def test_cost_split_balances_uneven_models():
    """Uneven models split by estimated cost (nodes x sweeps): every model once, and the
    largest share within 4/3 of the ideal (the longest-processing-time bound)."""
    import numpy as np
    rng = np.random.default_rng(5)
    grids = [(int(rng.integers(64, 257)), int(rng.integers(64, 257)), int(rng.integers(32, 129))) for _ in range(32)]
    costs = [sharding.field_cost(*g, sweeps=48) for g in grids]
    for world in (1, 2, 3, 8):
        parts = [sharding.shard_by_cost(costs, world, r) for r in range(world)]
        assert sorted(i for p in parts for i in p) == list(range(32))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= 4 / 3 * max(sum(costs) / world, max(costs)) + 1
    # equal costs reduce to a balanced count split
    parts = [sharding.shard_by_cost([7] * 10, 4, r) for r in range(4)]
    assert sorted(len(p) for p in parts) == [2, 2, 3, 3]
    with pytest.raises(ValueError):
        sharding.shard_by_cost(costs, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n_items, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r = sharding.world_rank()
        mine = list(range(n_items))[sharding.shard(n_items, w, r)]
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        costs = [(i * 7919) % 101 + 1 for i in range(n_items)]     # uneven fields
        by_cost = [None] * world
        dist.all_gather_object(by_cost, sharding.shard_by_cost(costs, w, r))
        sharding.barrier()
        step_ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
        slowest = sharding.max_over_ranks(step_ms)
        q.put((rank, gathered, slowest, by_cost, costs))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_sources_and_take_the_slowest_step():
    world, n_items = 2, 33
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_items, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, slowest, by_cost, costs in res:
        flat = [i for part in gathered for i in part]
        assert flat == list(range(n_items))       # disjoint, complete, in rank order
        assert slowest == 15.0                     # every rank sees the slowest rank's time
        # the cost split, computed by each rank alone, is one partition
        assert sorted(i for part in by_cost for i in part) == list(range(n_items))
        loads = [sum(costs[i] for i in part) for part in by_cost]
        assert max(loads) - min(loads) <= max(costs)
