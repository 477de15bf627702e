"""bench.py's multi-rank arithmetic on CPU: two gloo ranks (replicas of the workload).

Under torchrun every GPU runs its own replica of the batch; the reported time is the slowest
rank's and the value counts the units of all ranks.  The CUDA part of the bench needs a GPU; the
aggregation it uses is checked here with the gloo backend on 127.0.0.1.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], "cpu")
        v = bench.whole_job_rate(1000, world, t)
        dist.barrier()
        out.put((rank, t, v))
    finally:
        dist.destroy_process_group()


def test_two_ranks_slowest_time_and_whole_job_rate():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    times = [10.0, 25.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get() for _ in range(2))
    for rank, t, v in res:
        assert t == 25.0
        assert abs(v - 1000 * 2 / 0.025) < 1e-6


def test_single_process_is_its_own_maximum():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, "cpu") == 12.5
    assert bench.whole_job_rate(5952, 1, 40.0) == pytest.approx(148800.0)
