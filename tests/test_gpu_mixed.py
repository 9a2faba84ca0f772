"""Domains of several element types on the GPU (dnl_add_elements): the element pass, the lumped mass,
the Courant reduction and the Pulse power iteration run once per element group and assemble through
one node -> element-node map; so do the forward-mode tangents and the reverse-mode adjoint, on one
integration-point allocation in which each group has its block.

Against the reference's own outputs where the reference computes them soundly (tests/golden,
*mixed*): one force pass on an injected state of an ElTet4n3D + ElHex8n3D domain, and the lumped
mass, time steps and first steps of an ElTet4n3D + ElTet10n3D domain with the Courant step.  (The
reference's Pulse loop, and its force loop when a larger element precedes a smaller one, copy a
longer Vector into a shorter one on such domains -- Vector::redim, linearAlgebra/Vector.C:213-229 --
a heap overflow, so its hexahedron + tetrahedron runs pin nothing.)  The results file of an
ElTet4n3D + ElTet10n3D domain against the reference's own file.  The rest by identities: a
mesh split into two groups of its own element type runs bit for bit as the single group, and the
forces of a hexahedron + tetrahedron domain are those of its two parts as separate domains.
Gradients by identities and differences: the split mesh's tangents and adjoint are the single
group's bit for bit, the adjoint of a hexahedron + tetrahedron run is its forward-mode
contraction, and both match central differences of the scheduled run.  Tolerances as in
test_gpu_tets and test_gpu_sens."""

import dataclasses

import numpy as np
import pytest

from conftest import GOLDEN, golden
from oracle import states
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
STATE_TOL = 1e-12
TRAJ_TOL = 1e-7


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def tet_hex_bar():
    return meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D, upper=meshes.ELHEX8N3D)


def test_mixed_forces_injected_state_vs_reference(gpu_lib):
    """ElTet4n3D (first layer) + ElHex8n3D (two layers) in one domain, one computeInternalForces
    on the reference's injected mid-run state: forces and every integration point's new state."""
    g = golden("forces_mixed.npz")
    d = gpu_lib.GpuDomain(tet_hex_bar())
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"],
                v=st["v"], a=st["a"], disp=st["disp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=float(st["dt"]))
    assert rel(f, g["fint"]) <= FORCE_TOL
    out = d.get_state("S", "Eps", "EpsPlas", "p", "evp", "Sig")
    for k in out:
        assert rel(out[k], g["out_" + k]) <= STATE_TOL, k


def _two_materials():
    tx, ty = meshes.tabular_table(360e6, 316e6, 0.28)
    target = meshes.MaterialLaw(74.2e9, 0.33, 2784.0, meshes.HARD_TABULAR, (), tx, ty)
    copper = meshes.MaterialLaw(117e9, 0.35, 8930.0, meshes.HARD_POWER, (90e6, 292e6, 0.31))
    steel = meshes.MaterialLaw(193.6e9, 0.3, 7800.0, meshes.HARD_POWER, (250e6, 400e6, 0.4))
    return target, copper, steel


def test_mixed_two_materials_forces_vs_reference(gpu_lib):
    """The ElTet4n3D + ElHex8n3D domain of test_mixed_forces_injected_state_vs_reference with its
    tetrahedra of a tabular-hardening material and its hexahedra of a power-law one (materials
    and the element map over every group, dnl_set_materials after dnl_add_elements): one force pass
    on the reference's injected state, forces and every point's new state to 1e-12."""
    target, copper, _ = _two_materials()
    g = golden("forces_mixed_two.npz")
    d = gpu_lib.GpuDomain(meshes.group_materials(tet_hex_bar(), [target, copper]))
    st = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"],
                v=st["v"], a=st["a"], disp=st["disp"])
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=float(st["dt"]))
    assert rel(f, g["fint"]) <= FORCE_TOL
    out = d.get_state("S", "Eps", "EpsPlas", "p", "evp", "Sig")
    for k in out:
        assert rel(out[k], g["out_" + k]) <= STATE_TOL, k


def test_mixed_two_materials_steps_vs_reference(gpu_lib):
    """The ElTet4n3D + ElTet10n3D bar with its parts of two materials (other E, nu, rho and
    hardening), Courant: the lumped mass bit for bit (each element's density), the first time
    step bit for bit (each element's length over the sound speed of its own material and its
    nodes' densities, the interface nodes holding the last element's), then 3 steps: forces and
    times as in test_mixed_tet4_tet10_steps_vs_reference."""
    _, copper, steel = _two_materials()
    g = golden("steps_mixed_two.npz")
    d = gpu_lib.GpuDomain(meshes.group_materials(meshes.taylor_mixed(6, 12), [copper, steel]))
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(3):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k == 0 else TRAJ_TOL), k
        assert abs(d.time_info()["time"] - g["time"][k]) <= 1e-12 * g["time"][k], k
    assert rel(d.get_state("coords")["coords"], g["final_coords"]) <= TRAJ_TOL


def test_mixed_tet4_tet10_steps_vs_reference(gpu_lib):
    """ElTet4n3D (6 layers) + ElTet10n3D (6 layers), Courant: the lumped mass of both groups
    assembled bit for bit, the first time step bit for bit (the minimum of both groups' lengths
    over their sound speeds), then 5 steps: forces and time steps (the second step onwards from the
    ill-conditioned state ElTet10n3D's tables leave, as in test_tet10_mass_and_first_steps).  The
    forces stay within 1e-10 to 2e-9 of the reference's over the 5 steps; positions after them to
    the trajectory tolerance: the tables give some ElTet10n3D nodes negative lumped masses, whose
    accelerations turn those last-bit differences into 1.6e-8 of the coordinates."""
    g = golden("steps_mixed.npz")
    m = meshes.taylor_mixed(6, 12)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    assert rel(d.get_state("mass")["mass"], g["mass"][::3]) == 0.0
    assert d.time_step() == g["dt0"][0]
    for k in range(5):
        assert d.step(1) == 1
        assert rel(d.fint(), g["fint"][k]) <= (FORCE_TOL if k == 0 else TRAJ_TOL), k
        info = d.time_info()
        assert abs(info["time"] - g["time"][k]) <= 1e-12 * g["time"][k], k
    st = d.get_state("coords", "S", "p")
    assert rel(st["coords"], g["final_coords"]) <= TRAJ_TOL
    assert rel(st["S"], g["final_S"]) <= 1e-6
    assert rel(st["p"], g["final_p"]) <= 1e-6


@pytest.mark.parametrize("kind", ["hex_pulse", "tet4_courant", "hex_two_materials_pulse"])
def test_split_into_groups_is_bitwise_the_single_group(gpu_lib, kind):
    """A mesh given as two groups of its own element type (the first 40 % of its elements, then
    the rest through dnl_add_elements) numbers its element-node slots as the single group does, so
    every kernel sees the same data: 30 steps bit for bit (coordinates, forces, time, state); with
    two materials (tabular and elastic, Pulse) the groups read their elements' materials and Hooke
    entries from the one element map."""
    m = {"hex_pulse": lambda: meshes.taylor_hex(6, 8), "tet4_courant": lambda: meshes.taylor_tet(6, 8),
         "hex_two_materials_pulse": lambda: meshes.impact_two_materials_hex(4, 12)}[kind]()
    cut = int(0.4 * m.E)
    split = dataclasses.replace(m, conn=m.conn[:cut], groups=[(m.etype, m.conn[cut:])])
    a = gpu_lib.GpuDomain(m)
    b = gpu_lib.GpuDomain(split)
    assert a.step(30) == 30 and b.step(30) == 30
    sa, sb = a.get_state("coords", "v", "S", "evp"), b.get_state("coords", "v", "S", "evp")
    for k in ("coords", "v"):
        assert np.array_equal(sa[k], sb[k]), k
    for k in ("S", "evp"):
        assert np.array_equal(sa[k].reshape(-1), sb[k].reshape(-1)), k
    assert np.array_equal(a.fint(), b.fint())
    assert a.time_info()["time"] == b.time_info()["time"]


def test_hex_tet_forces_are_the_sum_of_both_parts(gpu_lib):
    """On a random mid-run state, the forces of the ElTet4n3D + ElHex8n3D domain equal those of its
    tetrahedra and of its hexahedra as two separate domains over the same nodes, to rounding (the
    mixed domain sums each node's slots in one pass, the sum of two domains adds two partial
    sums); the new integration-point states are the parts' own."""
    m = tet_hex_bar()
    st = states.random_state(m, seed=11)
    d = gpu_lib.GpuDomain(m)
    ip = dict(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    d.set_state(**ip)
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=st["dt"])
    out = d.get_state("S", "evp")
    n0 = m.E * m.nip  # integration points of the first group (tetrahedra, one each)
    parts, outs = [], []
    for (etype, conn), sl in zip(m.element_groups(), (slice(0, n0), slice(n0, None))):
        pm = dataclasses.replace(m, etype=etype, conn=conn, groups=None)
        p = gpu_lib.GpuDomain(pm)
        nip = meshes.NIP_OF[etype]
        p.set_state(**{k: v[sl].reshape((conn.shape[0], nip) + v.shape[1:]) for k, v in ip.items()})
        parts.append(p.internal_forces(coords=st["coords"], du=st["du"], dt=st["dt"]))
        outs.append(p.get_state("S", "evp"))
    assert rel(f, parts[0] + parts[1]) <= 1e-14
    for k in ("S", "evp"):
        whole = np.concatenate([o[k].reshape((-1,) + out[k].shape[1:]) for o in outs])
        assert np.array_equal(out[k], whole), k


def test_courant_step_takes_each_groups_sound_speed(gpu_lib):
    """Element::getSoundSpeed averages the element's nodal densities over its own node count, so
    with this density ElTet4n3D's and ElTet10n3D's speeds differ in the last bit; the Courant
    critical time is the minimum of every element's length over its own speed
    (Domain::computeCourantTimeStep), so the domain's first step is the smaller of its two parts'
    steps, bit for bit; and a graph-replayed run of the mixed domain is the stream-launched one."""
    m = meshes.taylor_mixed(4, 6, nz_lower=3, density=8930.0137)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    steps = []
    for etype, conn in m.element_groups():
        p = gpu_lib.GpuDomain(dataclasses.replace(m, etype=etype, conn=conn, groups=None))
        p.prologue()
        steps.append(p.time_step())
    assert d.time_step() == min(steps)
    a, b = gpu_lib.GpuDomain(m), gpu_lib.GpuDomain(m)
    assert a.step(4) == 4 and b.step_graph(4) == 4  # ElTet10n3D's tables: a few steps only
    assert np.array_equal(a.get_state("coords")["coords"], b.get_state("coords")["coords"])
    assert a.time_info()["time"] == b.time_info()["time"]


def test_hex_tet_bar_runs_with_pulse(gpu_lib):
    """The 6x6x12-cell bar, ElHex8n3D at the impact end and ElTet4n3D above, Pulse time step over
    both groups, 10 us of the impact: no error status, finite coordinates, and the same run bit
    for bit after dnl_reset on the same handle."""
    m = meshes.taylor_mixed(6, 12, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D, tend=10e-6)
    d = gpu_lib.GpuDomain(m)
    n = d.run()
    info = d.time_info()
    assert info["done"] == 1 and info["status"] == 0 and n > 10
    x1 = d.get_state("coords")["coords"]
    assert np.all(np.isfinite(x1))
    d.reset()
    assert d.run() == n
    assert np.array_equal(d.get_state("coords")["coords"], x1)


def test_failure_in_an_added_group_reports_the_domains_element_number(gpu_lib):
    """A flat ElTet4n3D (four nodes of the base plane: det J = 0) added after a bar's elements and
    a first added group: the element pass reports DNL_ERR_SINGULAR with that element's number in
    the domain (after every element before it), and the handle, reset, runs again."""
    t = meshes.taylor_tet(4, 3)
    base = t.bcs[0].nodes  # the z = 0 layer
    flat = np.array([[base[0], base[1], base[2], base[3]]], dtype=np.int64)
    d = gpu_lib.GpuDomain(t)
    d.add_elements(meshes.ELTET4N3D, t.conn[:5])
    d.add_elements(meshes.ELTET4N3D, flat)
    with pytest.raises(gpu_lib.DnlError) as err:
        d.internal_forces(coords=t.coords, du=np.zeros((t.N, 3)), dt=1e-8)
    assert err.value.code == 8 and err.value.element == t.E + 5


def test_add_elements_refusals(gpu_lib):
    """dnl_add_elements only before the run, only 3D reference elements of one family, ElHex8n3D
    only with the Pulse step, not on a batch's union mesh, not after several materials (they are
    set after the groups, over every group's elements); a batch does not take a domain of several
    types' state."""
    t = meshes.taylor_tet(4, 3)
    d = gpu_lib.GpuDomain(t)
    with pytest.raises(gpu_lib.DnlError):
        d.add_elements(meshes.ELHEX8N3D, meshes.taylor_hex(4, 3).conn[:2])  # Courant handle
    with pytest.raises(gpu_lib.DnlError):
        d.add_elements(meshes.ELQUA4NAX, np.zeros((1, 4), dtype=np.int64))  # another family
    d.add_elements(meshes.ELTET4N3D, t.conn[:3])
    with pytest.raises(ValueError):  # one material index per element of every group
        d.set_materials(t.material_laws() * 2, np.zeros(t.E, dtype=np.int64))
    d.set_materials(t.material_laws() * 2, np.r_[np.zeros(t.E), np.ones(3)].astype(np.int64))
    with pytest.raises(gpu_lib.DnlError):
        d.add_elements(meshes.ELTET4N3D, t.conn[:3])  # after several materials
    batch = gpu_lib.BatchDomain([t, t])
    with pytest.raises(gpu_lib.DnlError):
        batch.broadcast_state(d)
    view = batch.handle_view()
    c = np.ascontiguousarray(t.conn[:3], dtype=np.int32)
    assert gpu_lib.lib().dnl_add_elements(view.h, meshes.ELTET4N3D, 3, c.ctypes.data_as(gpu_lib._ip)) != 0
    d.step(2)
    with pytest.raises(gpu_lib.DnlError):
        d.add_elements(meshes.ELTET4N3D, t.conn[:3])  # after the run started
    a = gpu_lib.GpuDomain(meshes.taylor_axi(3, 4))
    with pytest.raises(gpu_lib.DnlError):
        a.add_elements(meshes.ELQUA4NAX, meshes.taylor_axi(3, 4).conn[:2])


def test_mixed_results_file_vs_reference_file(gpu_lib, tmp_path):
    """ElTet4n3D (2 layers) + ElTet10n3D (2 layers) after 2 steps, written by dnl_write_results,
    against the reference's Structure::writeData file of the same run (tests/golden,
    results_mixed.bin): each element's own integration points, elements in the domain's order;
    layout, headers, separators and time exactly, the mechanical fields per field to the
    trajectory tolerance of this domain's steps (test_mixed_tet4_tet10_steps_vs_reference).  The
    reference's file read into a fresh handle gives back its state exactly."""
    m = meshes.taylor_mixed(3, 4, nz_lower=2)
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    assert d.step(2) == 2
    path = str(tmp_path / "gpu.bin")
    d.write_results(path)
    ours = gpu_lib.parse_results(path, m.N, m.nIP_all)
    ref = gpu_lib.parse_results(f"{GOLDEN}/results_mixed.bin", m.N, m.nIP_all)
    for k in ("header", "domain_header", "thermal", "fe"):
        assert np.array_equal(ours[k], ref[k]), k
    for a, b in zip(ours["separators"], ref["separators"]):
        assert np.array_equal(a, b)
    assert abs(ours["time"] - ref["time"]) <= 1e-15 * ref["time"]
    errs = {k: rel(ours[k], ref[k]) for k in ("coords", "du", "disp", "v", "a", "S", "Sig", "Eps",
                                                "dEps", "EpsPlas", "p", "evp")}
    assert max(errs.values()) <= TRAJ_TOL, errs
    r = gpu_lib.GpuDomain(m)
    r.read_results(f"{GOLDEN}/results_mixed.bin")
    st = r.get_state("coords", "du", "v", "a", "disp", "S", "Eps", "EpsPlas", "p", "evp")
    for k in ("coords", "du", "v", "a", "disp", "p", "evp"):
        assert np.array_equal(np.ravel(st[k]), np.ravel(ref[k])), k
    # the handle keeps a symmetric tensor's upper triangle (the file's tensors can differ from
    # their transposes in the last bit)
    iu = np.triu_indices(3)
    for k in ("S", "Eps", "EpsPlas"):
        assert np.array_equal(st[k][:, iu[0], iu[1]], ref[k][:, iu[0], iu[1]]), k
    assert r.time_info()["time"] == ref["time"]


def test_mixed_restart_continues_the_run(gpu_lib, tmp_path):
    """The ElHex8n3D + ElTet4n3D bar with the Pulse step: a file written after 12 steps and read
    into a fresh handle gives back every group's state bit for bit (the file's per-point records
    against both handles' states) and the same next element pass to the parity tolerance (the
    cached evp^n is recomputed from evp on loading); the run then continues."""
    m = meshes.taylor_mixed(4, 8, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D)
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    assert d.step(12) == 12
    path = str(tmp_path / "w.bin")
    d.write_results(path)
    parsed = gpu_lib.parse_results(path, m.N, m.nIP_all)
    e = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    e.read_results(path)
    keys = ("coords", "du", "v", "a", "disp", "S", "Eps", "EpsPlas", "p", "evp")
    s1, s2 = d.get_state(*keys), e.get_state(*keys)
    for k in keys:
        assert np.array_equal(np.ravel(s1[k]), np.ravel(s2[k])), k
        assert np.array_equal(np.ravel(parsed[k]), np.ravel(s1[k])), k
    assert np.any(parsed["evp"] > 1e-10)  # the impact end is plastic
    x, du = s1["coords"], s1["du"]
    f1 = d.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    f2 = e.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    assert rel(f2, f1) <= FORCE_TOL
    assert e.step(10) == 10
    assert e.time_info()["status"] == 0
    assert np.all(np.isfinite(e.get_state("coords")["coords"]))


def plain_schedule(gpu_lib, m, nsteps):
    """The step sizes of the domain's own plain run (its Courant or Pulse estimate)."""
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    dts = []
    for _ in range(nsteps):
        dts.append(d.time_info()["time_step"])
        assert d.step(1) == 1
    return np.array(dts), d.get_state("coords")["coords"]


@pytest.mark.parametrize("kind", ["hex_pulse", "tet4_courant"])
def test_split_mesh_gradients_are_bitwise_the_single_groups(gpu_lib, kind):
    """The mesh given as two groups of its own element type: dnl_sens_run's final coordinates and
    tangents, and dnl_adjoint's gradient (its per-point parameter sums run over the points in
    element order either way), are those of the single group bit for bit."""
    m = meshes.taylor_hex(4, 8) if kind == "hex_pulse" else meshes.taylor_tet(4, 8)
    cut = int(0.4 * m.E)
    split = dataclasses.replace(m, conn=m.conn[:cut], groups=[(m.etype, m.conn[cut:])])
    dts, _ = plain_schedule(gpu_lib, m, 40)
    xa, dxa = gpu_lib.GpuDomain(m).sensitivities(dts)
    xb, dxb = gpu_lib.GpuDomain(split).sensitivities(dts)
    assert np.array_equal(xa, xb) and np.array_equal(dxa, dxb)
    assert np.all(np.abs(dxa).reshape(4, -1).max(axis=1) > 0)
    w = np.random.default_rng(5).normal(size=(m.N, 3))
    ga = gpu_lib.GpuDomain(m).adjoint(w, dts)
    gb = gpu_lib.GpuDomain(split).adjoint(w, dts)
    assert np.array_equal(ga, gb)


def hex_tet_gradient_bar():
    return meshes.taylor_mixed(4, 8, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D)


def test_mixed_sens_primal_is_the_plain_run(gpu_lib):
    """On the ElHex8n3D + ElTet4n3D bar, dnl_sens_run and dnl_run_schedule given the plain run's
    own step sizes are the plain run, bit for bit."""
    m = hex_tet_gradient_bar()
    dts, x_plain = plain_schedule(gpu_lib, m, 60)
    x, _ = gpu_lib.GpuDomain(m).sensitivities(dts)
    assert np.array_equal(x, x_plain)
    assert np.array_equal(gpu_lib.GpuDomain(m).run_schedule(dts), x_plain)


def test_mixed_reverse_mode_matches_forward_mode(gpu_lib):
    """The ElHex8n3D + ElTet4n3D bar, 60 scheduled steps (plastic at the impact end): dnl_adjoint
    with checkpoints, with kept and with regenerated per-point records, equals the forward-mode
    contraction (dx/dp)^T w to 1e-10 per parameter."""
    m = hex_tet_gradient_bar()
    dts, _ = plain_schedule(gpu_lib, m, 60)
    w = np.random.default_rng(3).normal(size=(m.N, 3))
    _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    ref = np.einsum("pnj,nj->p", dx, w)
    assert np.all(ref != 0.0)
    d = gpu_lib.GpuDomain(m)
    g = d.adjoint(w, dts, ckpt_stride=0)
    assert d.adjoint_stats()["kept_record_bytes"] > 0
    assert np.max(np.abs(g - ref) / np.abs(ref)) <= 1e-10, (g, ref)
    gpu_lib.set_adjoint_record_budget(0)
    try:
        e = gpu_lib.GpuDomain(m)
        g2 = e.adjoint(w, dts, ckpt_stride=8)
        assert e.adjoint_stats()["kept_record_bytes"] == 0
    finally:
        gpu_lib.set_adjoint_record_budget(2 << 30)
    assert np.array_equal(g, g2) or np.max(np.abs(g2 - ref) / np.abs(ref)) <= 1e-10


def test_mixed_tangents_match_central_differences(gpu_lib):
    """The forward-mode tangents of the ElHex8n3D + ElTet4n3D bar's final coordinates against
    central differences of the scheduled run (dnl_run_schedule, the same steps) at 1e-4 relative
    steps of A, B, n and |v0|: 1e-4 relative (2-norm) per parameter; a domain of several types
    takes a new material and speed through dnl_reset."""
    m = hex_tet_gradient_bar()
    dts, _ = plain_schedule(gpu_lib, m, 40)
    _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    d = gpu_lib.GpuDomain(m)
    base = np.array([m.A, m.B, m.n, np.linalg.norm(m.v0)])
    for p in range(4):
        h = 1e-4 * base[p]
        xs = []
        for sgn in (1.0, -1.0):
            q = base.copy()
            q[p] += sgn * h
            d.reset(gpu_lib.model_with_params(m, *q))
            xs.append(d.run_schedule(dts))
        fd = (xs[0] - xs[1]) / (2 * h)
        assert rel(dx[p], fd) <= 1e-4, (p, rel(dx[p], fd))


def test_mixed_torch_autograd_function(gpu_lib):
    """The torch.autograd.Function over a domain of several element types (the model's groups are
    added when its handle is made): the reverse-mode backward gives the forward-mode contraction
    of the same loss, and the forward-mode Function the same gradient."""
    torch = pytest.importorskip("torch")
    m = hex_tet_gradient_bar()
    dts, _ = plain_schedule(gpu_lib, m, 40)
    params = torch.tensor([m.A, m.B, m.n, float(np.linalg.norm(m.v0))], dtype=torch.float64,
                          requires_grad=True)
    target = torch.from_numpy(m.coords.copy())
    x = gpu_lib.taylor_autograd().apply(params, m, dts)
    ((x - target) ** 2).sum().backward()
    _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    ref = np.einsum("pnj,nj->p", dx, 2 * (x.detach().numpy() - m.coords))
    assert np.all(ref != 0.0)
    assert np.max(np.abs(params.grad.numpy() - ref) / np.abs(ref)) <= 1e-10
    pf = params.detach().clone().requires_grad_(True)
    ((gpu_lib.taylor_autograd("forward").apply(pf, m, dts) - target) ** 2).sum().backward()
    assert np.allclose(pf.grad.numpy(), ref, rtol=1e-12, atol=0)
