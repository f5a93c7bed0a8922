"""The multi-rank bookkeeping of bench.py (replicas: barrier, max over ranks, whole-job value) on
two gloo ranks on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    seconds = 1.0 + rank          # rank 1 is the slow replica
    m = bench.max_over_ranks(dist, seconds)
    v = bench.job_throughput(dist, world, 5, seconds)
    q.put((rank, m, v))
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == 2.0                 # max over ranks
        assert v == 2 * 5 / 2.0         # all ranks' units over the slowest time
