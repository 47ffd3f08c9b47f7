"""Multi-GPU policy: replicas only.

The reference's path has no exchange step on one device (its MPI domain
decomposition is disabled), and every box here has one GPU, so N GPUs run N
independent instances.  The only cross-rank operations are the bench's
timing reductions: the slowest rank's time and the total work.
"""
import torch
import torch.distributed as dist


def max_time_sum_units(elapsed_s: float, units: float):
    """(max over ranks of elapsed_s, sum over ranks of units)."""
    t = torch.tensor([elapsed_s], dtype=torch.float64)
    u = torch.tensor([float(units)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t, u = t.cuda(), u.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def shard_instances(n_instances: int, rank: int, world: int):
    """Instances of an ensemble owned by `rank` (round-robin, no data exchange)."""
    return list(range(rank, n_instances, world))
