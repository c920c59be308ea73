"""The N > 1 path of bench.py without GPUs: two gloo ranks on 127.0.0.1
reduce their step times with bench.max_over_ranks (the job time is the
slowest rank's) and report the whole-job value of bench.job_value; the
replicas exchange nothing else."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, dist)   # rank 1 is the slow one
    dist.barrier()
    q.put((rank, t, bench.job_value(world, 1000, t)))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    # 2 ranks x 1000 paths in 15 ms
    assert all(abs(o[2] - 2 * 1000 / 0.015) < 1e-6 for o in out)
