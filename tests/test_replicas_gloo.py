"""The multi-GPU path is replicas (one trajectory per rank, no collective on
the data path); its only exchange is the step-time reduction.  Checked here
with two gloo ranks on the CPU: every rank sees the slowest rank's time and
the job value counts every rank's pairs."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    step_ms = bench.slowest_rank(local_ms, dist)
    value = bench.job_throughput(1000, step_ms / 1e3, world)
    out[rank] = (step_ms, value)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_step():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        step_ms, value = res[r]
        assert step_ms == pytest.approx(150.0)
        assert value == pytest.approx(2 * 1000 / 0.150)
