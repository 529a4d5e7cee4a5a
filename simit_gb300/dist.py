"""Multi-process helpers: one process per GPU (torchrun environment), no
data-path collective.  Independent units (meshes of a batch) are sharded
across ranks; timings are reduced with a max over ranks."""
import os

import numpy as np


def env():
    """(rank, world, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_by_cost(costs, world):
    """Size-balanced greedy partition (longest processing time first): units
    in descending cost go to the currently lightest rank (lowest rank on
    ties).  Returns one ascending index list per rank; every unit is in
    exactly one."""
    costs = np.asarray(costs, np.float64)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    out = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        out[r].append(int(i))
        load[r] += costs[i]
    return [sorted(o) for o in out]


def max_over_ranks(value, device="cpu"):
    """Max of a float over all ranks of the default process group (the value
    itself when no group is initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device="cpu"):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
