"""The multi-rank (N > 1) benchmark path on the CPU: two gloo ranks, each with
its own seeded share of the workload, combined as the benchmark combines GPU
ranks (slowest rank's time, sum of the units), with no data-path exchange."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from geon_gb300 import shard
    alpha, lo, hi = bench.workload(shard.rank_seed(0x5EED, rank))
    units = 1000 * (rank + 1)
    t, u = shard.job_totals(dist, 1.5 + rank, units)
    dist.barrier()
    q.put((rank, float(alpha[:4].sum()), t, u))
    dist.destroy_process_group()


def test_two_rank_weak_scaling_totals():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a0, t0, u0), (r1, a1, t1, u1) = res
    assert (t0, u0) == (t1, u1) == (2.5, 3000)  # max of the times, sum of the units
    assert a0 != a1  # each rank traces its own share


def test_single_rank_totals_pass_through():
    from geon_gb300 import shard
    assert shard.job_totals(None, 0.25, 7) == (0.25, 7)
    assert shard.rank_seed(0x5EED, 3) == 0x5EED + 3
