"""Weak-scaling shards of the benchmark workloads across ranks.

Rays, bisection brackets and curvature points are independent, so each rank
(one process per GPU) traces its own seeded share and no data crosses ranks;
the only cross-rank operations are the barrier around the timed region and the
reduction of its result: the job's time is the slowest rank's, its work the sum
of every rank's.
"""
import torch


def rank_seed(base, rank):
    """Seed of a rank's share: distinct per rank, the same on every run."""
    return int(base) + int(rank)


def job_totals(dist, t_local, units_local, device="cpu"):
    """(time, units) of the whole job: max of the ranks' times, sum of their
    units. dist is torch.distributed (initialised) or None for one rank."""
    if dist is None:
        return float(t_local), int(units_local)
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(u)
    return float(t.item()), int(u.item())
