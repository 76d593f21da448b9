"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The hot path runs on one GPU per process; with N ranks each rank runs an
independent replica and the reported time is the maximum over ranks.  This
checks that aggregation and that the reference arm runs on rank 0 only,
without any GPU.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier_sync(dist)
        m = bench.max_over_ranks(dist, 10.0 + rank)

        class A:
            size = 16
            steps = 1
            warmup = 0
            ref_iters = 3
        ref = bench.bench_reference(A, rank, world, dist) if rank != 0 else "rank0"
        q.put((rank, m, ref))
        bench.barrier_sync(dist)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_rank0_only_reference():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res[0][1] == 11.0 and res[1][1] == 11.0      # max over ranks on every rank
    assert res[1][2] is None                             # rank 1 does no reference work
