"""Replica aggregation of the benchmark on two CPU ranks (gloo): every rank
times its own replica, the job's time is the slowest rank's, and the rate
counts the particles of all ranks."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    bench.barrier(w)
    ms_max = bench.max_over_ranks(ms, w)
    out[rank] = (r, w, local, ms_max, bench.replica_rate(1000, 10, ms_max, w))
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    port = free_port()
    ctx = mp.get_context("spawn")  # nothing forks a process that runs threads
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (r, w, local, ms_max, rate) in res.items():
        assert (r, w, local) == (rank, 2, rank)
        assert ms_max == 150.0
        assert rate == pytest.approx(2 * 1000 * 10 / 0.150)
