"""The N > 1 host path of bench.py on CPU: two gloo ranks each time their own
replica; the job time is the slowest rank's and the rate counts every rank's
timesteps (replicas only, no data-path collective)."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, value = bench.reduce_over_ranks(100.0 + 50.0 * rank, steps=200, world=world, device="cpu")
    r, w, _ = bench.dist_env()
    q.put((rank, ms, value, r, w))
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value, r, w in out:
        assert ms == pytest.approx(150.0)
        assert value == pytest.approx(2 * 200 / 0.150)
        assert (r, w) == (rank, 2)
