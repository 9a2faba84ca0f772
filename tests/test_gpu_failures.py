"""Failure statuses of the step, raised without faulting the GPU.

Every fatalError of the reference's path is a status code here.  The non-convergence statuses come
from loops with the reference's limits (29 Jacobi passes, Tensor2.C:1169-1258; 2000 Newton
iterations, Element.C:327-330; 1000 power iterations, Domain.C:936-939); dnl_set_iteration_caps
lowers a limit so that an ordinary small model reaches it, and the non-finite time step comes from a
material with zero density (infinite sound speed, zero Courant step).  Each case checks the status
and the element the library reports, through the single-mesh path (dnl_step / dnl_prologue) and,
where the batched path runs that model, through dnl_batch_step; then the same context runs a clean
model to the same bits as a fresh handle."""

import ctypes as C
import dataclasses

import numpy as np
import pytest

from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

RR_NOCONV, JACOBI_NOCONV, PULSE_NOCONV, ERR_DT = 2, 3, 4, 5


@pytest.fixture
def lib(gpu_lib):
    gpu_lib.set_iteration_caps()
    yield gpu_lib
    gpu_lib.set_iteration_caps()  # the reference's limits again


def _still_works(lib, d, m, steps=12):
    """After a failure: the same handle, reset, runs to the same bits as a fresh handle."""
    lib.set_iteration_caps()
    d.reset(m)
    d.prologue()
    d.step(steps)
    x = d.get_state("coords")["coords"]
    f = lib.GpuDomain(m)
    f.prologue()
    f.step(steps)
    xf = f.get_state("coords")["coords"]
    f.close()
    assert np.array_equal(x, xf)


def _batch_still_works(lib, b, models, steps=12):
    lib.set_iteration_caps()
    b.reset()
    b.prologue()
    b.step(steps)
    f = lib.BatchDomain(models)
    f.prologue()
    f.step(steps)
    for i in range(len(models)):
        assert np.array_equal(b.coords(i), f.coords(i))
    f.close()


def _batch_step_raw(b, n):
    act = C.c_int(0)
    rc = b.L.dnl_batch_step(b.h, int(n), C.byref(act))
    return rc, act.value


def test_jacobi_nonconvergence_single_mesh(lib):
    m = meshes.taylor_axi(1, 1)
    d = lib.GpuDomain(m)
    d.prologue()
    # a shear increment: the polar decomposition of F needs one rotation, which the cap of one
    # Jacobi pass (one check, then a rotation, no second check) leaves unconfirmed
    du = np.zeros((m.N, 3))
    du[:, 0] = 1e-3 * m.coords[:, 1]
    d.set_state(du=du)
    lib.set_iteration_caps(rotations=1)
    with pytest.raises(lib.DnlError) as ei:
        d.step(1)
    assert ei.value.code == JACOBI_NOCONV and ei.value.element == 0
    info = d.time_info()
    assert info["status"] == JACOBI_NOCONV and info["bad_element"] == 0
    _still_works(lib, d, m)


def test_jacobi_nonconvergence_batch(lib):
    models = [meshes.taylor_axi(2, 4), meshes.taylor_axi(3, 5, speed=200.0)]
    b = lib.BatchDomain(models)
    b.prologue()
    lib.set_iteration_caps(rotations=1)
    rc = 0
    for _ in range(60):  # until the radial expansion shears an element of each bar
        rc, _ = _batch_step_raw(b, 1)
        if all(b.time_info(i)["status"] for i in range(2)):
            break
    assert rc == JACOBI_NOCONV
    for i, mi in enumerate(models):
        info = b.time_info(i)
        assert info["status"] == JACOBI_NOCONV
        assert 0 <= info["bad_element"] < mi.E
    _batch_still_works(lib, b, models)


def test_radial_return_nonconvergence_single_mesh(lib):
    m = meshes.taylor_axi(1, 1)
    d = lib.GpuDomain(m)
    d.prologue()
    du = np.zeros((m.N, 3))
    du[:, 1] = -1e-2 * m.coords[:, 1]  # 1 % axial compression in one step: far past yield
    d.set_state(du=du)
    lib.set_iteration_caps(newton=0)
    with pytest.raises(lib.DnlError) as ei:
        d.step(1)
    assert ei.value.code == RR_NOCONV and ei.value.element == 0
    _still_works(lib, d, m)


def test_radial_return_nonconvergence_batch(lib):
    # a one-element bar at the nominal impact speed yields in its second step (the strain
    # increment is the previous step's displacement increment)
    models = [meshes.taylor_axi(1, 1), meshes.taylor_axi(1, 2, speed=150.0)]
    b = lib.BatchDomain(models)
    b.prologue()
    lib.set_iteration_caps(newton=0)
    rc = 0
    for _ in range(10):
        rc, _ = _batch_step_raw(b, 1)
        if all(b.time_info(i)["status"] for i in range(2)):
            break
    assert rc == RR_NOCONV
    for i, mi in enumerate(models):
        info = b.time_info(i)
        assert info["status"] == RR_NOCONV and 0 <= info["bad_element"] < mi.E
    _batch_still_works(lib, b, models)


def test_pulse_nonconvergence_single_mesh(lib):
    m = meshes.taylor_hex(4, 3)  # the Pulse time step (ElHex8n3D has no Courant length)
    d = lib.GpuDomain(m)
    lib.set_iteration_caps(power=1)
    with pytest.raises(lib.DnlError) as ei:
        d.prologue()
    assert ei.value.code == PULSE_NOCONV and ei.value.element == -1
    info = d.time_info()
    assert info["status"] == PULSE_NOCONV and info["bad_element"] == -1
    _still_works(lib, d, m, steps=6)


def test_nonfinite_time_step_single_mesh(lib):
    m = dataclasses.replace(meshes.taylor_axi(2, 3), density=0.0)  # infinite sound speed
    d = lib.GpuDomain(m)
    with pytest.raises(lib.DnlError) as ei:
        d.prologue()
    assert ei.value.code == ERR_DT and ei.value.element == -1
    ok = meshes.taylor_axi(2, 3)
    d.close()
    d = lib.GpuDomain(ok)
    _still_works(lib, d, ok)


def test_nonfinite_time_step_batch(lib):
    """One instance fails; the other keeps advancing in the same launches."""
    models = [meshes.taylor_axi(2, 3), dataclasses.replace(meshes.taylor_axi(2, 4), density=0.0)]
    b = lib.BatchDomain(models)
    rc = b.L.dnl_batch_prologue(b.h)
    assert rc == ERR_DT
    assert b.time_info(0)["status"] == 0
    info = b.time_info(1)
    assert info["status"] == ERR_DT and info["bad_element"] == -1
    rc, active = _batch_step_raw(b, 5)
    assert rc == ERR_DT
    assert b.time_info(0)["increment"] == 5 and b.time_info(1)["increment"] == 0
    # instance 0 advanced exactly as alone
    alone = lib.GpuDomain(models[0])
    alone.prologue()
    alone.step(5)
    assert np.array_equal(b.coords(0), alone.get_state("coords")["coords"])
    alone.close()
