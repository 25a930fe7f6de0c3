"""bench.py's multi-rank arithmetic with two gloo ranks on CPU: every rank
gets the slowest rank's step time and the job throughput counts every
replica's samples (replicas only: beams are independent, no data exchange)."""
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
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(1.0 + rank)   # rank 0: 1 ms, rank 1: 2 ms
    q.put((rank, ms, bench.job_throughput(world, ms), bench._dist()))
    dist.destroy_process_group()


def test_max_over_ranks_and_throughput_gloo_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for rank, ms, value, (ws, r) in res:
        assert ms == 2.0 and ws == 2 and r == rank
        assert value == pytest.approx(2 * bench.BEAMS * bench.N_POINT / 2e-3 / 1e6)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_throughput(1, 1.0) == pytest.approx(bench.BEAMS * bench.N_POINT / 1e-3 / 1e6)
