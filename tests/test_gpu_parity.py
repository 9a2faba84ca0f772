"""Parity of the CUDA path (through the C ABI) with the reference outputs (tests/golden) and the
oracle.  Tolerances, from the specification of this path:

* nodal internal forces of one step from the same state: relative 2-norm error <= 1e-12
* integration-point state after that step: relative 2-norm error <= 1e-12 per field
* final nodal positions after a full run: max |dx| / max |x| <= 1e-6
"""

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


def _state_from_golden(g):
    return {k[3:]: g[k] for k in g.files if k.startswith("in_")}


@pytest.mark.parametrize("name,model", [("forces_axi.npz", lambda: meshes.taylor_axi(3, 4)),
                                        ("forces_hex.npz", lambda: meshes.taylor_hex(4, 3))])
def test_internal_forces_injected_state(gpu_lib, name, model):
    """dnl_internal_forces on a mid-run state vs the reference's Domain::computeInternalForces."""
    g = golden(name)
    m = model()
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    st = _state_from_golden(g)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"],
                v=st["v"], a=st["a"], disp=st["disp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=float(st["dt"]))
    assert rel(f, g["fint"]) <= FORCE_TOL
    out = d.get_state("S", "Eps", "EpsPlas", "p", "evp", "Sig")
    for k in ("S", "Eps", "EpsPlas", "p", "evp", "Sig"):
        assert rel(out[k], g["out_" + k]) <= STATE_TOL, k
    dE, R = d.step_tensors()
    assert rel(dE, g["out_dEps"]) <= STATE_TOL
    assert rel(R, g["out_R"]) <= STATE_TOL


@pytest.mark.parametrize("etype,seed", [(0, 11), (1, 12), (0, 13), (1, 14)])
def test_internal_forces_random_states_vs_oracle(gpu_lib, etype, seed):
    m = meshes.taylor_axi(12, 40) if etype == 0 else meshes.taylor_hex(10, 12)
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


def test_steps_c0_per_step_forces(gpu_lib):
    """The 5x50 Taylor bar: each of the first 20 steps' Fint, dt and kinetic energy."""
    g = golden("steps_c0.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_axi(5, 50))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::2]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(20):
        assert d.step(1) == 1
        f = d.fint()
        r = g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert rel(f, r) <= FORCE_TOL, k
        info = d.time_info()
        assert abs(info["time"] - g["time"][k]) <= 1e-15 * g["time"][k]
        assert abs(info["kinetic"] - g["kinetic"][k]) <= 1e-12 * g["kinetic"][k]


def test_full_run_c0_final_positions(gpu_lib):
    """5x50 Taylor impact to 80 us: final positions within 1e-6 of the reference."""
    g = golden("run_c0.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_axi(5, 50))
    n = d.run()
    info = d.time_info()
    assert info["done"] == 1 and info["status"] == 0
    assert abs(n - int(g["increments"][0])) <= 2
    x = d.get_state("coords")["coords"].ravel()
    ref = g["final_coords"]
    err = np.max(np.abs(x - ref)) / np.max(np.abs(ref))
    assert err <= POS_TOL, err
    evp = d.get_state("evp")["evp"].ravel()
    assert rel(evp, g["final_evp"]) <= 1e-6


def test_runs_are_bitwise_deterministic(gpu_lib):
    m = meshes.taylor_axi(10, 100)
    out = []
    for _ in range(2):
        d = gpu_lib.GpuDomain(m)
        d.step(300)
        out.append((d.get_state("coords")["coords"], d.fint()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_graph_replay_equals_stream_steps(gpu_lib):
    m = meshes.taylor_axi(8, 60)
    a = gpu_lib.GpuDomain(m)
    a.step(60)
    b = gpu_lib.GpuDomain(m)
    b.prologue()
    for _ in range(3):
        assert b.step_graph(20) == 20
    assert np.array_equal(a.get_state("coords")["coords"], b.get_state("coords")["coords"])
    assert a.time_info()["time"] == b.time_info()["time"]


def test_multi_step_vs_oracle_taylor_fine(gpu_lib):
    """A finer axi bar (20x200) for 200 steps: positions and plastic strain vs the oracle."""
    m = meshes.taylor_axi(20, 200)
    o = Oracle(m)
    o.prologue()
    o.steps(200)
    d = gpu_lib.GpuDomain(m)
    assert d.step(200) == 200
    x = d.get_state("coords")["coords"].ravel()
    assert np.max(np.abs(x - o.array("coords"))) <= 1e-12 * np.max(np.abs(o.array("coords")))
    assert rel(d.fint(), o.array("fint")) <= 1e-10


def test_negative_jacobian_is_reported(gpu_lib):
    """An inverted element gives DNL_ERR_NEG_DETJ with its index; the context stays usable."""
    m = meshes.taylor_axi(3, 3)
    d = gpu_lib.GpuDomain(m)
    x = m.coords.copy()
    e = 4
    n0, n2 = m.conn[e, 0], m.conn[e, 2]
    x[[n0, n2]] = x[[n2, n0]]
    with pytest.raises(gpu_lib.DnlError) as ei:
        d.internal_forces(coords=x, du=np.zeros((m.N, 3)))
    assert ei.value.code == 1
    f = d.internal_forces(coords=m.coords, du=np.zeros((m.N, 3)))
    assert np.all(np.isfinite(f))


def test_steps_hex_pulse(gpu_lib):
    """6x6x8 hex bar with the Pulse time step, 30 steps along the trajectory vs the reference.

    The 3D polar decomposition picks its Jacobi pivot by comparing |C_01|, |C_02|, |C_12|; on the
    bar's diagonal planes two of them are equal up to rounding, and it stops at |C_pq| < 1e-9, so a
    last-bit difference upstream selects another rotation path whose result differs at that
    tolerance.  The reference itself shows this: its restatement built with fused multiply-adds
    (GCC's default on aarch64) departs from the x86 build by 1e-9 at step 3 and 1.4e-8 by step 30
    on this bar.  So the trajectory is held to 1e-7 per step (the first steps to 1e-12), and single
    steps from identical states to 1e-12 (test_internal_forces_*).  The Pulse time step is a power
    iteration stopped at a 1e-4 change of its estimate; its products K x are formed matrix-free and
    summed in another order than the reference's assembled Ke, so dt and time agree to 1e-10."""
    g = golden("steps_hex.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_hex(6, 8))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-10 * g["dt0"][0]
    for k in range(30):
        assert d.step(1) == 1
        r = g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert rel(d.fint(), r) <= (FORCE_TOL if k < 3 else 1e-7), k
        info = d.time_info()
        assert abs(info["time"] - g["time"][k]) <= 1e-10 * g["time"][k]
    x = d.get_state("coords")["coords"].ravel()
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-9 * np.max(np.abs(g["final_coords"]))


def test_full_run_hex_final_positions(gpu_lib):
    """8x8x24 hex bar, Pulse time step, to 80 us (2873 increments): final positions <= 1e-6."""
    g = golden("run_hex.npz")
    d = gpu_lib.GpuDomain(meshes.taylor_hex(8, 24))
    n = d.run()
    assert d.time_info()["done"] == 1
    assert abs(n - int(g["increments"][0])) <= 2
    x = d.get_state("coords")["coords"].ravel()
    err = np.max(np.abs(x - g["final_coords"])) / np.max(np.abs(g["final_coords"]))
    assert err <= POS_TOL, err


def test_imposed_speed_bar_vs_reference(gpu_lib):
    """The tensile bar pulled by BoundarySpeed (Boundary.C:478-525) on one end and clamped by
    BoundaryRestrain 1 1 1 on the other, Pulse time step, against the reference's own outputs:
    lumped mass bitwise, the imposed velocity exact on the pulled nodes, the first 2 steps' forces
    to 1e-12, the next 28 to 1e-6, positions after 30 steps to 1e-9; then the bar pulled at 5 m/s to
    2 ms (373 increments, plastic): final positions <= 1e-6.

    Why not 1e-12 all along: pulled at 1 m/s, the wave front carries strains of order 1e-9, where
    the polar decomposition's Jacobi stop (|C_pq| < 1e-9) decides whether a point rotates at all, so
    a last-bit difference in F flips that decision and the step's forces move by ~1e-9.  The
    reference shows it against itself: its restatement built with fused multiply-adds (the
    reference's own rounding on aarch64) departs from its x86 build by 1.3e-13 at step 2, 1.5e-9 at
    step 3 and 2.3e-7 by step 30 on this bar, with positions 3e-11 apart after 30 steps and 2e-15
    after the full run.  The GPU follows the same profile; one element pass from the GPU's own
    state at steps 2, 3, 5, 10 and 20 agrees with the oracle to <= 7e-13."""
    g = golden("steps_speed.npz")
    m = meshes.necking_bar(4, 12)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert abs(d.time_step() - g["dt0"][0]) <= 1e-10 * g["dt0"][0]
    for k in range(30):
        assert d.step(1) == 1
        r = g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert rel(d.fint(), r) <= (FORCE_TOL if k < 2 else 1e-6), k
        info = d.time_info()
        assert abs(info["time"] - g["time"][k]) <= 1e-10 * g["time"][k]
    st = d.get_state("coords", "v")
    x = st["coords"].ravel()
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-9 * np.max(np.abs(g["final_coords"]))
    top = m.bcs[1].nodes
    assert np.array_equal(st["v"][top, 2], np.full(top.size, 1.0))
    r = golden("run_speed.npz")
    d = gpu_lib.GpuDomain(meshes.necking_bar(4, 12, speed=5.0, tend=2e-3))
    n = d.run()
    assert d.time_info()["done"] == 1
    assert abs(n - int(r["increments"][0])) <= 2
    x = d.get_state("coords")["coords"].ravel()
    err = np.max(np.abs(x - r["final_coords"])) / np.max(np.abs(r["final_coords"]))
    assert err <= POS_TOL, err


def test_imposed_speed_pass_from_gpu_state_vs_oracle(gpu_lib):
    """One element pass of the imposed-speed bar from the GPU's own state at steps 3 and 10 (the
    pulled end's Current delta_disp = v dt, the wave front just past the Jacobi stop's scale), in
    the GPU and in the oracle: 1e-12 on the forces."""
    m = meshes.necking_bar(4, 12)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    done = 0
    for k in (2, 9):
        d.step(k - done)
        done = k
        st = d.get_state("coords", "du", "S", "Eps", "EpsPlas", "p", "evp")
        dt = d.time_info()["time_step"]
        o = Oracle(m)
        o.prologue()
        o.inject(coords=st["coords"], du=st["du"], v=np.zeros((m.N, 3)), a=np.zeros((m.N, 3)),
                 disp=np.zeros((m.N, 3)), S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"],
                 p=st["p"], evp=st["evp"], dt=dt)
        o.internal_matrices()
        fo = o.internal_forces()
        p = gpu_lib.GpuDomain(m)
        p.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
        fg = p.internal_forces(coords=st["coords"], du=st["du"], dt=dt)
        p.close()
        assert rel(fg, fo) <= FORCE_TOL, (k, rel(fg, fo))


def test_pulse_time_step_vs_oracle_medium(gpu_lib):
    """A 16x16x40 hex bar: the Pulse step after the prologue and after 25 steps vs the oracle."""
    m = meshes.taylor_hex(16, 40)
    o = Oracle(m)
    o.prologue()
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    assert abs(d.time_step() - o.get("dt")) <= 1e-10 * o.get("dt")
    o.steps(25)
    d.step(25)
    assert abs(d.time_step() - o.get("dt")) <= 1e-10 * o.get("dt")
    x = d.get_state("coords")["coords"].ravel()
    assert np.max(np.abs(x - o.array("coords"))) <= 1e-9 * np.max(np.abs(o.array("coords")))


def test_profile_counts_kernels(gpu_lib):
    d = gpu_lib.GpuDomain(meshes.taylor_axi(5, 50))
    d.prologue()
    d.profile_begin()
    d.step(10)
    prof = d.profile_end()
    assert prof["elem"][1] == 10 and prof["node"][1] == 10
    assert prof["elem"][0] > 0.0
