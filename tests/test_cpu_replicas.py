"""Replica aggregation of bench.py over two gloo ranks on the CPU (the path --gpus N takes)."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from waves_gb300.replicas import aggregate
    # rank r simulated (r + 1) * 0.5 s in (r + 1) * 2 s of device time, e2e 0.25 s in 3 + r s
    got = aggregate((rank + 1) * 0.5, (rank + 1) * 2.0, 0.25, 3.0 + rank)
    out[rank] = got
    dist.destroy_process_group()


def test_two_rank_aggregate():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        sim, dev, e2e_sim, e2e_wall = out[rank]
        assert sim == pytest.approx(1.5) and dev == pytest.approx(4.0)
        assert e2e_sim == pytest.approx(0.5) and e2e_wall == pytest.approx(4.0)


def test_single_process_passthrough():
    from waves_gb300.replicas import aggregate
    assert aggregate(1.0, 2.0, 3.0, 4.0) == (1.0, 2.0, 3.0, 4.0)
