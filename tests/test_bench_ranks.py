"""bench.py's multi-GPU path on the CPU: two gloo ranks (replicas) agree on the job time
(the slowest rank's) and on the whole-job throughput (both ranks' iterations)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        local_ms = [120.0, 150.0][rank]
        total, value = bench.job_throughput(local_ms, steps=10, world=world, dist=dist, device="cpu")
        out[rank] = (total, value)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    total, value = res[0]
    assert total == 150.0
    assert value == pytest.approx(2 * 10 / 0.150)


def test_single_rank_needs_no_collective():
    import bench
    total, value = bench.job_throughput(200.0, steps=4, world=1)
    assert total == 200.0 and value == pytest.approx(20.0)
