"""World-size-2 gloo test of the replica policy's host logic (CPU only)."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from hydrothermal3d_gb300.replicas import max_time_sum_units, shard_instances
    t, u = max_time_sum_units(1.0 + rank, 10.0 * (rank + 1))
    mine = shard_instances(7, rank, world)
    q.put((rank, t, u, mine))
    dist.barrier()
    dist.destroy_process_group()


def test_max_time_sum_units_two_ranks():
    import random
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + random.randint(0, 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, u, mine in res:
        assert t == 2.0 and u == 30.0
    assert res[0][3] == [0, 2, 4, 6] and res[1][3] == [1, 3, 5]
