"""The replicated (N > 1) bench path on CPU: world_size-2 gloo ranks, each with its own
timing, agree on the slowest rank's time, and the job's throughput counts every
replica's cells.  The step itself has no collective (replicas only)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    out.put((rank, bench.max_over_ranks(ms, world), bench.job_throughput(1000, 3, 4, world, bench.max_over_ranks(ms, world) / 1e3)))
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 3 * 1000 * 4 * 2 / 0.015) < 1e-6 for r in res)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(10, 3, 2, 1, 0.5) == 120.0
