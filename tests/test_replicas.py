"""The N > 1 path of bench.py: independent replicas, one per rank, no
collective on the data path; the job time is the slowest rank's and the
throughput counts every rank's particles.  Run as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = [10.0, 40.0][rank]
        n_local = [1000, 3000][rank]
        value, ms = bench.aggregate(ms_local, n_local, 5, world, dist)
        out.put((rank, value, ms))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
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
    for rank, value, ms in res:
        assert ms == 40.0
        assert value == pytest.approx((1000 + 3000) * 5 / 0.040)
