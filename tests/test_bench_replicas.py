"""The multi-GPU path of bench.py is replicas only: each rank transforms
its own grid and the job's time is the slowest rank's.  These tests run the
bench's reduction and aggregation with world size 2 over gloo on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    assert bench.replica_env() == (world, rank, rank)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
    t = bench.max_over_ranks(torch, dist, ms, torch.device("cpu"))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, bench.aggregate_gpts(world, 1 << 30, t)))


def test_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [15.0, 15.0]
    # two replicas of 2^30 points in 15 ms
    assert res[0][2] == pytest.approx(2 * (1 << 30) / 15e-3 / 1e9)


def test_single_process_needs_no_collective():
    import bench
    torch = pytest.importorskip("torch")
    assert bench.max_over_ranks(torch, None, 3.5, torch.device("cpu")) == 3.5
    assert bench.aggregate_gpts(1, 10 ** 9, 1000.0) == pytest.approx(1.0)
