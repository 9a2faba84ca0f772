"""Batched mode (dnl_batch_*): many uneven axisymmetric Taylor bars advanced together must give,
instance by instance, exactly what the single-mesh path gives -- the kernels and their arithmetic
are the same, only the launch covers all instances."""

import numpy as np
import pytest

from oracle.oracle import Oracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu


def _models():
    return [meshes.taylor_axi(4, 40, speed=180.0, A=70e6, B=250e6, n=0.25),
            meshes.taylor_axi(7, 60, speed=260.0, A=120e6, B=380e6, n=0.45),
            meshes.taylor_axi(5, 50),
            meshes.taylor_axi(10, 45, speed=150.0, A=60e6, B=200e6, n=0.2)]


def test_batch_matches_single_meshes_bitwise(gpu_lib):
    models = _models()
    b = gpu_lib.BatchDomain(models)
    b.prologue()
    assert b.step(120) == len(models)
    for i, m in enumerate(models):
        d = gpu_lib.GpuDomain(m)
        assert d.step(120) == 120
        assert np.array_equal(b.coords(i), d.get_state("coords")["coords"]), i
        assert np.array_equal(b.fint(i), d.fint()), i
        assert b.time_info(i)["time"] == d.time_info()["time"]


def test_batch_graph_and_autotune_keep_results(gpu_lib):
    models = _models()
    a = gpu_lib.BatchDomain(models)
    a.step(60)
    b = gpu_lib.BatchDomain(models)
    blk = b.autotune(steps=4)  # 2 modes x 3 block sizes x (1 untimed + 4 timed) = 30 steps
    assert blk in (64, 128, 256)
    assert b.tuning() in {(mode, blk) for mode in (gpu_lib.BATCH_LAUNCHES, gpu_lib.BATCH_PERSISTENT)}
    for _ in range(3):
        b.step_graph(10)
    for i in range(len(models)):
        assert np.array_equal(a.coords(i), b.coords(i)), i


def test_persistent_step_matches_launch_sequence(gpu_lib):
    """One persistent cooperative kernel per step (grid barriers between the phases) gives the
    launch sequence's results bit for bit, stream-launched and graph-replayed, with every block
    size; so it also equals each bar run alone."""
    models = _models()
    ref = gpu_lib.BatchDomain(models)
    ref.step(70)
    for block in (64, 128, 256):
        b = gpu_lib.BatchDomain(models)
        b.set_mode(gpu_lib.BATCH_PERSISTENT)
        b.set_block(block)
        assert b.tuning() == (gpu_lib.BATCH_PERSISTENT, block)
        b.step(30)
        b.step_graph(20)
        b.step_graph(20)
        for i in range(len(models)):
            assert np.array_equal(ref.coords(i), b.coords(i)), (block, i)
            assert np.array_equal(ref.fint(i), b.fint(i)), (block, i)
            assert ref.time_info(i)["time"] == b.time_info(i)["time"], (block, i)
        b.close()


@pytest.mark.parametrize("mode", ["launches", "persistent"])
def test_batch_runs_each_instance_to_its_end(gpu_lib, mode):
    """Two small bars with different end times: each stops at its own end time; final positions
    vs the oracle within the full-run tolerance."""
    m1 = meshes.taylor_axi(4, 40, tend=6e-6)
    m2 = meshes.taylor_axi(5, 50, speed=200.0, tend=9e-6)
    b = gpu_lib.BatchDomain([m1, m2])
    b.set_mode(gpu_lib.BATCH_PERSISTENT if mode == "persistent" else gpu_lib.BATCH_LAUNCHES)
    active = 2
    while active:
        active = b.step(200)
    for i, m in enumerate((m1, m2)):
        info = b.time_info(i)
        assert info["done"] == 1 and abs(info["time"] - m.tend) <= 1e-15 * m.tend
        o = Oracle(m)
        o.prologue()
        o.steps(10 ** 9)
        x = b.coords(i).ravel()
        ref = o.array("coords")
        assert np.max(np.abs(x - ref)) <= 1e-6 * np.max(np.abs(ref))


def test_graph_capture_then_replay(gpu_lib):
    """dnl_batch_graph_capture prepares the graph without advancing; the replays that follow give
    what stream launches give."""
    models = _models()
    a = gpu_lib.BatchDomain(models)
    a.step(40)
    b = gpu_lib.BatchDomain(models)
    b.prologue()
    b.graph_capture(20)
    for i in range(len(models)):
        assert b.time_info(i)["increment"] == 0
    b.step_graph(20)
    b.step_graph(20)
    for i in range(len(models)):
        assert np.array_equal(a.coords(i), b.coords(i)), i


def test_full_size_batch_matches_single_meshes_bitwise(gpu_lib):
    """The benchmark's batch at full size (256 seeded uneven bars, 1.28 M elements, autotuned block,
    graph-replayed steps): a sample of instances, the smallest and largest among them, equal bit
    for bit to the same bars run alone after 40 steps."""
    models = meshes.taylor_batch(256, seed=0)
    b = gpu_lib.BatchDomain(models)
    b.prologue()
    b.autotune(steps=3)
    b.reset()
    b.prologue()
    b.step_graph(20)
    b.step_graph(20)
    sizes = [m.E for m in models]
    sample = sorted({0, 37, 101, 200, 255, int(np.argmin(sizes)), int(np.argmax(sizes))})
    for i in sample:
        d = gpu_lib.GpuDomain(models[i])
        assert d.step(40) == 40
        assert np.array_equal(b.coords(i), d.get_state("coords")["coords"]), i
        assert np.array_equal(b.fint(i), d.fint()), i
        assert b.time_info(i)["time"] == d.time_info()["time"], i
        d.close()
