"""Multi-process (replicas-only) aggregation of bench.py on CPU with the gloo backend, world size 2:
each rank's value is combined by max (time) and sum (rays), exactly what rank 0 reports."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as td

    import bench

    td.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(td, 10.0 + rank)       # per-rank time
    r = bench.reduce_sum(td, 100.0 * (rank + 1))  # per-rank rays
    bench.barrier(td)
    q.put((rank, t, r))
    td.destroy_process_group()


def test_bench_replica_aggregation_gloo():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp

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
    assert res == [(0, 11.0, 300.0), (1, 11.0, 300.0)]
    del torch
