"""The multi-rank (N > 1) benchmark path on the CPU: two gloo ranks, each with
its own seeded share of the workload, combined as the benchmark combines GPU
ranks (slowest rank's time, sum of the units), with no data-path exchange."""
import os
import socket

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


def _rank_end_to_end(rank, world, port, q):
    """One rank of the benchmark's multi-rank path, end to end on the CPU: the
    rank's own seeded workload (bench.rank_workload), a trace of a small sample
    of it (the CPU oracle stands in for the GPU stepper), the barrier, and the
    reduction of time and units bench.main uses (shard.job_totals)."""
    import time

    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle as orc
    alpha, lo, hi = bench.rank_workload(rank)
    sample = alpha[:16]
    dist.barrier()
    t0 = time.perf_counter()
    term, steps = orc.shadow_classify(bench.SCHW, bench.R_OBS, sample, 0.05, 4000, math=orc.LIBM, nthreads=1)
    dt = time.perf_counter() - t0
    t, u = bench.shard_totals(dist, dt, int(steps.sum()))
    dist.barrier()
    q.put((rank, sample.tolist(), dt, int(steps.sum()), t, u))
    dist.destroy_process_group()


def test_two_rank_benchmark_path_end_to_end():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_end_to_end, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, dt0, n0, t0, u0), (r1, s1, dt1, n1, t1, u1) = res
    assert s0 != s1  # per-rank seeds: each rank traces its own share
    assert (t0, u0) == (t1, u1)  # every rank sees the job's totals
    assert t0 == max(dt0, dt1) and u0 == n0 + n1 > 0  # slowest rank's time, sum of the work
    import bench
    assert bench.rank_workload(0)[0][:16].tolist() == s0  # rank 0's share is the single-GPU workload


def test_single_rank_totals_pass_through():
    from geon_gb300 import shard
    assert shard.job_totals(None, 0.25, 7) == (0.25, 7)
    assert shard.rank_seed(0x5EED, 3) == 0x5EED + 3
