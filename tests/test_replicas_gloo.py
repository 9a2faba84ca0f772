"""The multi-GPU mode of bench.py is independent replicas: no collective on the data path, only a
barrier and the max of the per-rank times.  Checked here with two gloo ranks on the CPU (127.0.0.1
rendezvous): each rank reports its own time, every rank gets the maximum."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        bench.barrier(w)
        t = bench.barrier_and_max(10.0 + 5.0 * r, w)
        q.put((r, w, local, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[3] == 15.0 for g in got)
