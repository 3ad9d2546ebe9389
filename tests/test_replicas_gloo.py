"""Multi-GPU runs are replicas (the path has no exchange step): the host-side aggregation of
bench.py, run as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [100.0, 125.0][rank]
    local_units = [1e9, 1e9][rank]
    value, max_ms = bench.replica_throughput(local_ms, local_units, dist, "cpu")
    out[rank] = (value, max_ms)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        value, max_ms = out[r]
        assert max_ms == 125.0
        assert abs(value - 2e9 / 0.125) < 1e-6 * value


def test_single_process():
    import bench
    assert bench.replica_throughput(50.0, 1e8) == (2e9, 50.0)
