"""The plane-strain quad (ElQua4n2D: ElementPlane's F with no hoop stretch, no 2 pi R weight, no
hoop force) on the GPU, against the reference's own outputs (tests/golden, *_plane*) and the
oracle.  Tolerances are those of the axisymmetric and 3D paths: 1e-12 relative on one step's
forces and state from the same inputs, 1e-6 on the final positions of a full run."""

import dataclasses

import numpy as np
import pytest

from conftest import golden
from oracle import states
from oracle.oracle import Oracle, SensOracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
STATE_TOL = 1e-12
POS_TOL = 1e-6
SENS_TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def test_plane_forces_injected_state_vs_reference(gpu_lib):
    g = golden("forces_plane.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_plane(3, 4), flags=gpu_lib.FLAG_STEP_TENSORS)
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"],
                v=st["v"], a=st["a"], disp=st["disp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=float(st["dt"]))
    assert rel(f, g["fint"]) <= FORCE_TOL
    out = d.get_state("S", "Eps", "EpsPlas", "p", "evp", "Sig")
    for k in out:
        assert rel(out[k], g["out_" + k]) <= STATE_TOL, k
    dE, R = d.step_tensors()
    assert rel(dE, g["out_dEps"]) <= STATE_TOL
    assert rel(R, g["out_R"]) <= STATE_TOL


@pytest.mark.parametrize("seed", [31, 32])
def test_plane_forces_random_states_vs_oracle(gpu_lib, seed):
    m = meshes.taylor_plane(12, 40)
    st = states.random_state(m, seed=seed)
    o = Oracle(m)
    o.inject(**st)
    o.internal_matrices()
    fo = o.internal_forces()
    d = gpu_lib.GpuDomain(m)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=st["dt"])
    assert rel(f, fo) <= FORCE_TOL
    out = d.get_state("S", "EpsPlas", "evp", "p")
    for k in out:
        assert rel(out[k], o.array(k)) <= STATE_TOL, k


def test_plane_steps_vs_reference(gpu_lib):
    """The 5x50 plane-strain bar: lumped mass, first time step, each of 40 steps' forces."""
    g = golden("steps_plane.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_plane(5, 50))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::2]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(40):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k < 20 else 1e-11), k
        info = d.time_info()
        assert abs(info["kinetic"] - g["kinetic"][k]) <= 1e-12 * g["kinetic"][k]


def test_plane_full_run_vs_reference(gpu_lib):
    g = golden("run_plane.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_plane(5, 50))
    n = d.run()
    info = d.time_info()
    assert info["done"] == 1 and info["status"] == 0
    assert abs(n - int(g["increments"][0])) <= 2
    x = d.get_state("coords")["coords"].ravel()
    err = np.max(np.abs(x - g["final_coords"])) / np.max(np.abs(g["final_coords"]))
    assert err <= POS_TOL, err
    assert rel(d.get_state("evp")["evp"], g["final_evp"]) <= 1e-6


def test_plane_pulse_vs_reference(gpu_lib):
    g = golden("steps_plane_pulse.npz")
    d = gpu_lib.GpuDomain(dataclasses.replace(meshes.taylor_plane(5, 50), method=meshes.PULSE))
    d.prologue()
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-12 * g["dt0"][0]
    for k in range(30):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= 1e-11, k
    x = d.get_state("coords")["coords"].ravel()
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-12 * np.max(np.abs(g["final_coords"]))


def test_plane_batch_matches_single_meshes_bitwise(gpu_lib):
    models = [meshes.taylor_plane(4, 40, speed=180.0, A=70e6, B=250e6, n=0.25),
              meshes.taylor_plane(7, 60, speed=260.0),
              meshes.taylor_plane(5, 50)]
    b = gpu_lib.BatchDomain(models)
    b.prologue()
    assert b.step(100) == len(models)
    for i, m in enumerate(models):
        d = gpu_lib.GpuDomain(m)
        assert d.step(100) == 100
        assert np.array_equal(b.coords(i), d.get_state("coords")["coords"]), i
        assert np.array_equal(b.fint(i), d.fint()), i


def test_plane_sensitivities_vs_dual_oracle(gpu_lib):
    m = meshes.taylor_plane(5, 50)
    o = Oracle(m)
    o.prologue()
    dts = []
    for _ in range(300):
        dts.append(o.get("dt"))
        o.steps(1)
    dts = np.array(dts)
    s = SensOracle(m, mass=o.array("mass").copy())
    s.run(dts)
    xo, dxo = s.coords()
    x, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    assert np.max(np.abs(x - xo)) <= 1e-12 * np.max(np.abs(xo))
    for p in range(4):
        assert np.linalg.norm(dxo[p]) > 0
        assert rel(dx[p], dxo[p]) <= SENS_TOL, (p, rel(dx[p], dxo[p]))
