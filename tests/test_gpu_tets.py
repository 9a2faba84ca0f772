"""The tetrahedra on the GPU: ElTet4n3D (one Gauss point, Courant length = shortest edge) and
ElTet10n3D (four points; the reference's tables as they evaluate, see oracle/dnl_oracle.c
tet10_tables), against the reference's own outputs (tests/golden, *tet*) and the oracle.
Tolerances as for the hexahedron: 1e-12 relative on one step's forces and state from the same
inputs; along a trajectory 1e-12 for the first steps, then 1e-7 (the 3D Jacobi rotation chooses its
pivot by comparing |C_01|, |C_02|, |C_12|, which are equal up to rounding on symmetry planes of
the bar, so a last-bit difference upstream can select another rotation path whose result differs
at its 1e-9 stopping tolerance -- see test_steps_hex_pulse); 1e-6 on the final positions of a full
run."""

TRAJ_TOL = 1e-7

import dataclasses

import numpy as np
import pytest

from conftest import golden
from oracle import states
from oracle.oracle import Oracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
STATE_TOL = 1e-12
POS_TOL = 1e-6


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


@pytest.mark.parametrize("name,quadratic", [("forces_tet4.npz", False), ("forces_tet10.npz", True)])
def test_tet_forces_injected_state_vs_reference(gpu_lib, name, quadratic):
    g = golden(name)
    d = gpu_lib.GpuDomain(meshes.taylor_tet(4, 3, quadratic=quadratic),
                          flags=gpu_lib.FLAG_STEP_TENSORS)
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


# ElTet4n3D only: the reference's ElTet10n3D Jacobian J = sum_k x_k dN_k/dxi picks up
# (sum_k dN_k/dxi) x, which is not zero for its tables, so it depends on where the element sits and
# can be nearly singular; random states then reach strain increments of 1 to 7 in one step, where
# ln U of a nearly singular F is ill-conditioned (agreement ~1e-6 at a few points).  Its parity is
# pinned by the reference's own injected-state fixture above.
@pytest.mark.parametrize("seed", [41, 43])
def test_tet4_forces_random_states_vs_oracle(gpu_lib, seed):
    m = meshes.taylor_tet(8, 12)
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


def test_tet4_steps_vs_reference(gpu_lib):
    g = golden("steps_tet4.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_tet(6, 8))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(40):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k < 2 else TRAJ_TOL), k
        info = d.time_info()
        assert abs(info["kinetic"] - g["kinetic"][k]) <= 1e-9 * g["kinetic"][k]


def test_tet4_full_run_vs_reference(gpu_lib):
    g = golden("run_tet4.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_tet(6, 8))
    n = d.run()
    info = d.time_info()
    assert info["done"] == 1 and info["status"] == 0
    assert abs(n - int(g["increments"][0])) <= 2
    x = d.get_state("coords")["coords"].ravel()
    err = np.max(np.abs(x - g["final_coords"])) / np.max(np.abs(g["final_coords"]))
    assert err <= POS_TOL, err
    assert rel(d.get_state("evp")["evp"], g["final_evp"]) <= 1e-6


def test_tet4_pulse_vs_reference(gpu_lib):
    g = golden("steps_tet4_pulse.npz")
    d = gpu_lib.GpuDomain(dataclasses.replace(meshes.taylor_tet(6, 8), method=meshes.PULSE))
    d.prologue()
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-12 * g["dt0"][0]
    for k in range(20):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k < 2 else TRAJ_TOL), k


def test_tet10_mass_and_first_steps_vs_reference(gpu_lib):
    """The reference's run of this element blows up after two steps (negative lumped corner
    masses, derivative tables that do not sum to zero); those two steps agree, the second -- from
    the ill-conditioned state the first leaves -- to the trajectory tolerance."""
    g = golden("steps_tet10.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_tet(6, 8, quadratic=True))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(2):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k == 0 else TRAJ_TOL), k
    x = d.get_state("coords")["coords"].ravel()
    assert rel(x, g["final_coords"]) <= 1e-9


def test_tet4_batch_matches_single_meshes_bitwise(gpu_lib):
    models = [meshes.taylor_tet(4, 6, speed=180.0), meshes.taylor_tet(6, 8),
              meshes.taylor_tet(5, 7, speed=260.0, A=120e6)]
    b = gpu_lib.BatchDomain(models)
    b.prologue()
    assert b.step(60) == len(models)
    for i, m in enumerate(models):
        d = gpu_lib.GpuDomain(m)
        assert d.step(60) == 60
        assert np.array_equal(b.coords(i), d.get_state("coords")["coords"]), i
        assert np.array_equal(b.fint(i), d.fint()), i
