"""The multi-GPU form of the bench is replicas: each rank runs its own
pattern, the job time is the slowest rank's and the work the sum over ranks.
This checks that aggregation with two gloo ranks on the CPU (no GPU, no
data-path collective)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [100.0, 250.0][rank]      # rank 1 is the slowest
        local_units = [1000, 3000][rank]
        value, ms = bench.replica_throughput(local_ms, local_units, dist, device="cpu")
        out[rank] = (value, ms)
    finally:
        dist.destroy_process_group()


def test_two_rank_replica_throughput():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        value, ms = out[r]
        assert ms == 250.0                   # the slowest rank's time
        assert abs(value - 4000 / 0.25) < 1e-6   # all units over that time


def test_single_rank_replica_throughput():
    import bench
    value, ms = bench.replica_throughput(50.0, 500)
    assert ms == 50.0 and abs(value - 10000.0) < 1e-9
