"""Hardening laws other than the power law and several materials per mesh on the GPU
(dnl_set_materials), against the reference's own outputs (tests/golden, generated from the
compiled reference): a two-material impact in the pattern of Samples/Traction/Traction.dyn
(tabular-hardening target, projectile without hardening carrying its own initial velocity), the
same pair on a hexahedral bar with the Pulse time step, and the Taylor bar with an IsoHardMetafor
law.  One element pass from identical (injected) states within
the per-step tolerance (1e-12 relative 2-norm); along the 40-step trajectories the forces of the
first 20 steps within 1e-12 and of the next 20 within 1e-11 (the few-ulp differences of each pass
accumulate); the lumped mass exactly, the first step size to 1e-12."""

import numpy as np
import pytest

from conftest import golden
from oracle.oracle import Oracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name,model", [("steps_two.npz", lambda: meshes.impact_two_materials(5, 50)),
                                        ("steps_metafor.npz", lambda: meshes.metafor_bar(5, 50))])
def test_laws_and_materials_vs_reference(gpu_lib, name, model):
    g = golden(name)
    m = model()
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    assert np.array_equal(d.get_state("mass")["mass"], g["mass"][::2])
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-12 * g["dt0"][0]
    for k in range(40):
        assert d.step(1) == 1
        if np.linalg.norm(g["fint"][k]) > 0:
            assert rel(d.fint(), g["fint"][k]) <= (TOL if k < 20 else 10 * TOL), k
    assert rel(d.get_state("coords")["coords"], g["final_coords"]) <= TOL
    assert rel(d.get_state("evp")["evp"], g["final_evp"]) <= 1e-10


@pytest.mark.parametrize("model,seed", [(lambda: meshes.impact_two_materials(8, 40), 21),
                                        (lambda: meshes.metafor_bar(8, 40), 22)])
def test_laws_single_pass_from_identical_states(gpu_lib, model, seed):
    """One dnl_internal_forces from a random mid-run state (the same injected into the oracle,
    which is bit-exact with the reference for these laws): forces and state within 1e-12."""
    from oracle import states
    m = model()
    st = states.random_state(m, seed=seed)
    o = Oracle(m)
    o.inject(**st)
    o.internal_matrices()
    fo = o.internal_forces()
    d = gpu_lib.GpuDomain(m)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=st["dt"])
    assert rel(f, fo) <= TOL
    out = d.get_state("S", "EpsPlas", "evp", "p")
    for k in out:
        assert rel(out[k], o.array(k)) <= TOL, k
    assert np.max(o.array("evp") - st["evp"].ravel()) > 0  # some points yielded in this pass


def test_two_materials_longer_run_vs_oracle(gpu_lib):
    """400 steps of the two-material impact: positions vs the oracle (its restatement is bit-exact
    with the reference over the first 40)."""
    m = meshes.impact_two_materials(5, 50)
    d = gpu_lib.GpuDomain(m)
    assert d.step(400) == 400
    o = Oracle(m)
    o.prologue()
    o.steps(400)
    x = d.get_state("coords")["coords"].ravel()
    ref = o.array("coords")
    assert np.max(np.abs(x - ref)) <= 1e-9 * np.max(np.abs(ref))


def test_two_materials_hex_pulse_vs_reference(gpu_lib):
    """The two bonded materials on a 4x4x12-cell ElHex8n3D bar with the Pulse time step, whose
    power iteration forms K x with each element's own Hooke matrix (Element3D.C:242-333 reads the
    element's material): lumped mass bit for bit, the first step size and the times to 1e-10 (the
    power iteration sums K x in another order than the reference's assembled Ke), forces of the
    first 2 steps to 1e-12 and of the next 28 to 1e-7 (3D Jacobi pivot ties and stopping tests, as
    in test_steps_hex_pulse: here the third step's forces are 1.3e-11 away with the time steps
    equal to 5e-16, the fifth's 1.4e-8), final positions to 1e-9; the tabular target yields."""
    g = golden("steps_two_hex.npz")
    m = meshes.impact_two_materials_hex(4, 12)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    assert np.array_equal(d.get_state("mass")["mass"], g["mass"][::3])
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-10 * g["dt0"][0]
    for k in range(30):
        assert d.step(1) == 1
        if np.linalg.norm(g["fint"][k]) > 0:
            assert rel(d.fint(), g["fint"][k]) <= (TOL if k < 2 else 1e-7), k
        assert abs(d.time_info()["time"] - g["time"][k]) <= 1e-10 * g["time"][k], k
    x = d.get_state("coords")["coords"].ravel()
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-9 * np.max(np.abs(g["final_coords"]))
    assert d.get_state("evp")["evp"].max() > 1e-3


def test_material_arguments_are_checked(gpu_lib):
    m = meshes.impact_two_materials(3, 10)
    d = gpu_lib.GpuDomain(meshes.taylor_axi(3, 10))
    laws = m.material_laws()
    with pytest.raises(gpu_lib.DnlError):  # several materials need an element map
        d.set_materials(laws, None)
    bad = np.full(m.E, 2)
    with pytest.raises(gpu_lib.DnlError):  # index out of range
        d.set_materials(laws, bad)
    d.prologue()
    with pytest.raises(gpu_lib.DnlError):  # after the prologue
        d.set_materials(laws, m.elem_material)
    s = gpu_lib.GpuDomain(m)
    with pytest.raises(gpu_lib.DnlError):  # sensitivities need one power-law material
        s.sensitivities(np.full(5, 1e-9))
