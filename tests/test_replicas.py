"""The multi-GPU mode of bench.py is replicas only (no data-path collective):
every rank runs the whole workload and the job's time is the slowest rank's.
This checks that reduction with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.replica_throughput(100.0 + 50.0 * rank, 1000, 4, world, torch.device("cpu"))
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            ms, value = out[r]
            assert ms == 150.0
            assert abs(value - 1000 * 4 * 2 / 0.150) < 1e-6
