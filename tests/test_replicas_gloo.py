"""The multi-GPU mode of bench.py is independent replicas: each rank advances its own copy of the
workload with no collective on the data path; only a barrier, the max of the per-rank times and the
sum of the units processed cross ranks.  Checked here with two gloo ranks on the CPU (127.0.0.1
rendezvous), the oracle standing in for each rank's device: each rank reports its own time and
every rank gets the maximum; the whole-job rate is the summed units over the slowest rank's time;
and each rank, given the same workload, advances it to the same state a single process reaches."""

import os
import socket

import numpy as np
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
    from oracle.oracle import Oracle
    from redynela_gb300 import meshes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        bench.barrier(w)
        t = bench.barrier_and_max(10.0 + 5.0 * r, w)
        rate = bench.aggregate_rate(100.0 * (r + 1), 2.0 + r, w)
        # this rank's replica: its own copy of the workload, advanced on its own
        o = Oracle(meshes.taylor_axi(3, 12), threads=1)
        o.prologue()
        done = o.steps(25)
        q.put((r, w, local, t, rate, done, o.array("coords").copy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_are_independent_replicas():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.oracle import Oracle
    from redynela_gb300 import meshes
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted((q.get(timeout=120) for _ in range(2)), key=lambda g: g[0])
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert [g[2] for g in got] == [0, 1]  # each rank on its own local device index
    assert all(g[3] == 15.0 for g in got)  # the max of 10 and 15
    assert all(abs(g[4] - 300.0 / 3.0) < 1e-12 for g in got)  # (100 + 200) units / max(2, 3) s
    o = Oracle(meshes.taylor_axi(3, 12), threads=1)
    o.prologue()
    assert o.steps(25) == 25
    for g in got:
        assert g[5] == 25
        assert np.array_equal(g[6], o.array("coords"))
