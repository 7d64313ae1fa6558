"""The replica path of bench.py --gpus N on the CPU: two gloo ranks take the
element-wise maximum of their step times (the slowest replica defines the
job's time) and pass the barriers."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench._dist = dist
    bench.barrier(world)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 3.5], world)
    bench.barrier(world)
    out[rank] = got
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1] == [2.0, 10.0, 3.5]


def test_single_rank_is_a_pass_through():
    import bench
    assert bench.max_over_ranks([1.25, 2.5], 1) == [1.25, 2.5]
