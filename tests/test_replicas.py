"""bench.py with N > 1: replicas (each rank its own workload), the whole-job
value over the slowest rank's time.  Two gloo ranks on the CPU exercise the
same aggregation the NCCL run uses."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r "took" 10 + 5 r ms for its replica of 2e12 flops
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, torch.device("cpu"))
    value = bench.aggregate_value(2e12, world, ms)
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_and_sum_the_work():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # every rank sees the slowest rank's time, and the value counts both replicas
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 15.0
    assert value == pytest.approx(2 * 2e12 / 15e-3)
