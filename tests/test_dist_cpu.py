"""The multi-process path on CPU: two gloo ranks (torchrun-style
environment, rendezvous on 127.0.0.1).  Checks the size-balanced sharding of
a batch of meshes (every sheet on exactly one rank, loads within 10 %), the
max/sum reductions used for timing, and that the reference arm prints from
rank 0 only."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from simit_gb300 import dist as sgd
    from simit_gb300 import problems
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = sgd.env()
    sides = problems.cloth_sides(256)
    shard = sgd.shard_by_cost(sides.astype(np.float64) ** 2, w)[r]
    shards = [None] * w
    dist.all_gather_object(shards, shard)
    mx = sgd.max_over_ranks(10.0 + r)
    sm = sgd.sum_over_ranks(float(len(shard)))
    # the reference arm: rank 0 alone runs and prints (tiny sample)
    import bench
    args = type("A", (), {"warmup": 0, "steps": 1, "cpu_sample": 3, "size": 128,
                           "no_reorder": False})()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args, r, w)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, shards, mx, sm, buf.getvalue()))


def test_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = res[0][1]
    assert shards == res[1][1]
    allidx = sorted(i for s in shards for i in s)
    assert allidx == list(range(256))
    from simit_gb300 import problems
    cost = problems.cloth_sides(256).astype(np.float64) ** 2
    loads = [cost[s].sum() for s in shards]
    assert max(loads) <= 1.1 * (sum(loads) / world)
    assert all(r[2] == 11.0 for r in res)
    assert all(r[3] == 256.0 for r in res)
    out0 = res[0][4].strip().splitlines()
    assert len(out0) == 1 and json.loads(out0[0])["impl"] == "reference"
    assert json.loads(out0[0])["n_gpus"] == 2
    assert res[1][4].strip() == ""


def test_shard_by_cost_single_rank_and_ties():
    from simit_gb300 import dist as sgd
    assert sgd.shard_by_cost([3, 1, 2], 1) == [[0, 1, 2]]
    s = sgd.shard_by_cost([5, 5, 5, 5], 2)
    assert sorted(s[0] + s[1]) == [0, 1, 2, 3] and len(s[0]) == len(s[1]) == 2
