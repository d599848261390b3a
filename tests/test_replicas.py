"""The multi-GPU path of bench.py is replicas only: every rank solves its own
problem and the job reports the slowest rank's time with the summed work.
The aggregation runs here as two gloo ranks on CPU."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev_s = [1.5, 2.0][rank]
        wall_s = [1.7, 2.4][rank]
        iters = [50, 47][rank]
        out[rank] = bench.aggregate_replicas(torch, dist, dev_s, wall_s, iters, "cpu")
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
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
        res = dict(out)
    assert res[0] == res[1] == (2.0, 2.4, 97.0)


def test_single_process_passes_through():
    assert bench.aggregate_replicas(torch, None, 1.25, 1.5, 50, "cpu") == (1.25, 1.5, 50)
