"""The multi-GPU form of the benchmark is replicas only (rays are independent, the grid is
read-only): each rank renders its own frame and the job's rate is all ranks' rays over the
slowest rank's time.  The reduction and the rate run here as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 1.0 + 0.5 * rank  # the second rank is slower
        slowest = bench.max_over_ranks(ms, "cpu")
        out[rank] = (bench.dist_env(), slowest, bench.replica_rate(1000, slowest * 1e-3, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in (0, 1):
        env, slowest, rate = out[r]
        assert env == (r, r, 2)
        assert slowest == 1.5
        assert rate == pytest.approx(2 * 1000 / 1.5e-3)
