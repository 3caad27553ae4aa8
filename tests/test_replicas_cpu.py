"""The multi-GPU path of bench.py is replicas only (independent problems,
no data-path collective): the job rate is world_size problems per step of
the slowest replica.  Checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r timed 100 (r + 1) ms over 10 steps
        rate, total = bench.replica_rate(100.0 * (rank + 1), 10)
        q.put((rank, rate, total))
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    import multiprocessing as mp
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
    # slowest replica: 200 ms for 10 steps -> 20 ms per step, two problems per step
    for _, rate, total in out:
        assert total == pytest.approx(200.0)
        assert rate == pytest.approx(2 / 0.020)


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    rate, total = bench.replica_rate(250.0, 10)
    assert total == 250.0 and rate == pytest.approx(1 / 0.025)
