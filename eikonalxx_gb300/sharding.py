"""Sources across processes, one process per GPU.

The path shards into independent units, one travel-time field per source, so a multi-GPU
job is a set of replicas. Each rank solves its own share -- a contiguous slice of equal
fields (sources on one model), or a split by estimated cost of fields of uneven size
(models of different grids) -- and no collective touches the data path. The only
collectives are the timing barrier and the max-over-ranks reduction of the step time.
"""
import os


def world_rank():
    """(world size, rank) from the launcher's environment (torchrun sets both)."""
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def shard(n_items, world, rank):
    """Contiguous slice of `n_items` for `rank` out of `world`; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def field_cost(nx, ny, nz, sweeps):
    """Estimated cost of one field: node updates, nodes x sweeps (the sweep kernels are
    bound by node updates once a launch is full)."""
    return int(nx) * int(ny) * int(nz) * int(sweeps)


def shard_by_cost(costs, world, rank):
    """Indices of the items `rank` solves out of `world`, split by estimated cost: the
    items are dealt, most expensive first, to the rank with the least cost so far (ties to
    the lower rank) -- the longest-processing-time rule, whose largest share is within 4/3
    of the best split.  Deterministic, so every rank computes the same split without a
    collective; each rank's indices are returned in ascending order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0] * world
    owner = [0] * len(costs)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value, device=None):
    """Largest `value` over all ranks (the job's step time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
