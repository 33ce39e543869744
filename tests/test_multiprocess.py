"""The N > 1 host path of bench.py on CPU: two gloo ranks, max-over-ranks
timing and the replica throughput rule (value = all ranks' DoFs / slowest
rank's time).  Multi-GPU runs are independent replicas (one operator per GPU),
so there is no data-path collective to test."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), MFGB_BENCH_BACKEND="gloo")
    import bench
    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slowest
    bench.barrier(w)
    worst = bench.max_over_ranks(ms, w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((rank, worst))


def test_two_rank_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_replica_throughput_rule():
    import bench
    n_dofs, world, worst_ms = 67634433, 4, 3.9
    value = world * n_dofs / (worst_ms * 1e-3) / 1e9
    assert value == pytest.approx(4 * 67634433 / 3.9e-3 / 1e9)
    assert bench.max_over_ranks(2.5, 1) == 2.5
