"""The oracle (oracle/dnl_oracle.c) against the reference's own outputs (tests/golden, generated by
tests/golden/make_golden.py from the compiled reference) and against known answers.  CPU only."""

import dataclasses

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as orc
from oracle.oracle import Oracle
from redynela_gb300 import meshes


def _inject(o, g):
    o.inject(**{k[3:]: (g[k] if k != "in_dt" else float(g[k])) for k in g.files if k.startswith("in_")})


def test_tables_match_reference():
    g = golden("tables.npz")
    for et, nm in ((0, "axi"), (1, "hex"), (2, "plane"), (3, "tet4"), (4, "tet10")):
        N, dN = orc.tables(et)
        assert np.array_equal(N.ravel(), g[nm + "_N"])
        assert np.array_equal(dN.ravel(), g[nm + "_dN"])
    for nm, w in (("axi", 1.0), ("hex", 1.0), ("plane", 1.0), ("tet4", 1. / 6.), ("tet10", 1.0 / 24.0)):
        assert np.all(g[nm + "_weight"] == w)
    # the reference's ElTet10n3D derivative tables do not sum to zero over the nodes (two negated
    # constants are unparenthesised macros): the oracle reproduces that, it is not a mistake here
    dN10 = g["tet10_dN"].reshape(4, 10, 3)
    assert np.all(np.abs(dN10.sum(axis=1)) > 1.7)
    assert np.all(np.abs(g["tet4_dN"].reshape(1, 4, 3).sum(axis=1)) == 0.0)


@pytest.mark.parametrize("name,model", [("forces_axi.npz", lambda: meshes.taylor_axi(3, 4)),
                                        ("forces_hex.npz", lambda: meshes.taylor_hex(4, 3)),
                                        ("forces_plane.npz", lambda: meshes.taylor_plane(3, 4)),
                                        ("forces_tet4.npz", lambda: meshes.taylor_tet(4, 3)),
                                        ("forces_tet10.npz",
                                         lambda: meshes.taylor_tet(4, 3, quadratic=True))])
def test_internal_forces_bit_exact(name, model):
    """One Domain::computeInternalForces on an injected mid-run state: bit for bit."""
    g = golden(name)
    m = model()
    o = Oracle(m)
    _inject(o, g)
    o.internal_matrices()
    f = o.internal_forces()
    assert np.array_equal(f, g["fint"])
    for k in ("S", "Eps", "EpsPlas", "p", "evp", "Sig", "dEps", "R"):
        assert np.array_equal(o.array(k), g["out_" + k]), k
    # the state exercises both branches of the radial return
    assert np.any(o.array("evp") != g["in_evp"].ravel())
    assert np.any(o.array("evp") == g["in_evp"].ravel())


def test_steps_c0_bit_exact():
    g = golden("steps_c0.npz")
    o = Oracle(meshes.taylor_axi(5, 50))
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert o.get("dt") == g["dt0"][0]
    for k in range(20):
        assert o.get("dt") == g["dt"][k] or k == 0
        o.steps(1)
        assert np.array_equal(o.array("fint"), g["fint"][k]), k
        assert o.get("kinetic_current") == g["kinetic"][k]
        assert o.get("time") == g["time"][k]
    assert np.array_equal(o.array("coords"), g["final_coords"])


def test_run_c0_bit_exact():
    """The full 5x50 Taylor run to 80 us (9722 increments) reproduces the reference bit for bit."""
    g = golden("run_c0.npz")
    o = Oracle(meshes.taylor_axi(5, 50))
    o.prologue()
    n = o.steps(10 ** 9)
    assert n == int(g["increments"][0])
    assert o.get("time") == g["time"][0]
    assert np.array_equal(o.array("coords"), g["final_coords"])
    assert np.array_equal(o.array("evp"), g["final_evp"])
    assert np.array_equal(o.array("S"), g["final_S"])


def test_plane_strain_steps_and_run_bit_exact():
    """ElQua4n2D (ElementPlane: no hoop stretch, no 2 pi R weight, no hoop force): 40 steps with
    their forces, then the full run to 80 us, bit for bit with the reference."""
    g = golden("steps_plane.npz")
    m = meshes.taylor_plane(5, 50)
    o = Oracle(m)
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert o.get("dt") == g["dt0"][0]
    for k in range(40):
        o.steps(1)
        assert np.array_equal(o.array("fint"), g["fint"][k]), k
        assert o.get("kinetic_current") == g["kinetic"][k]
    assert np.array_equal(o.array("coords"), g["final_coords"])
    assert np.array_equal(o.array("S"), g["final_S"])
    g = golden("run_plane.npz")
    o = Oracle(m)
    o.prologue()
    assert o.steps(10 ** 9) == int(g["increments"][0])
    assert o.get("time") == g["time"][0]
    assert np.array_equal(o.array("coords"), g["final_coords"])
    assert np.array_equal(o.array("evp"), g["final_evp"])
    assert g["final_evp"].max() > 1.0


def test_tet4_steps_and_run_bit_exact():
    """ElTet4n3D (one point, Courant length = shortest edge): 40 steps, then the full run."""
    g = golden("steps_tet4.npz")
    m = meshes.taylor_tet(6, 8)
    o = Oracle(m)
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert o.get("dt") == g["dt0"][0]
    for k in range(40):
        o.steps(1)
        assert np.array_equal(o.array("fint"), g["fint"][k]), k
    assert np.array_equal(o.array("coords"), g["final_coords"])
    g = golden("run_tet4.npz")
    o = Oracle(m)
    o.prologue()
    assert o.steps(10 ** 9) == int(g["increments"][0])
    assert np.array_equal(o.array("coords"), g["final_coords"])
    assert np.array_equal(o.array("evp"), g["final_evp"])


def test_tet4_pulse():
    g = golden("steps_tet4_pulse.npz")
    o = Oracle(dataclasses.replace(meshes.taylor_tet(6, 8), method=meshes.PULSE))
    o.prologue()
    assert abs(o.get("dt") - g["dt0"][0]) <= 1e-14 * g["dt0"][0]
    for k in range(20):
        o.steps(1)
        r = g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert np.linalg.norm(o.array("fint") - r) <= 1e-12 * np.linalg.norm(r), k


def test_tet10_mass_and_first_steps_bit_exact():
    """ElTet10n3D: the lumped mass (negative at the corner nodes: row sums of the quadratic shape
    functions) and the two steps the reference's run of this bar survives."""
    g = golden("steps_tet10.npz")
    o = Oracle(meshes.taylor_tet(6, 8, quadratic=True))
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert np.any(g["mass"] < 0)
    assert o.get("dt") == g["dt0"][0]
    for k in range(2):
        o.steps(1)
        assert np.array_equal(o.array("fint"), g["fint"][k]), k
    assert np.array_equal(o.array("coords"), g["final_coords"])


def test_steps_plane_pulse():
    """ElQua4n2D with the Pulse time step (plane-strain Hooke matrix, Material.C:276-284)."""
    g = golden("steps_plane_pulse.npz")
    o = Oracle(dataclasses.replace(meshes.taylor_plane(5, 50), method=meshes.PULSE))
    o.prologue()
    assert abs(o.get("dt") - g["dt0"][0]) <= 1e-14 * g["dt0"][0]
    for k in range(30):
        o.steps(1)
        f, r = o.array("fint"), g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert np.linalg.norm(f - r) <= 1e-12 * np.linalg.norm(r), k
    x = o.array("coords")
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-12 * np.max(np.abs(g["final_coords"]))


def test_steps_hex_pulse():
    """Hex8 with the Pulse time step: the power iteration sums K.x in element order where the
    reference uses its Jobs order, so agreement is to rounding, not bitwise."""
    g = golden("steps_hex.npz")
    o = Oracle(meshes.taylor_hex(6, 8))
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert abs(o.get("dt") - g["dt0"][0]) <= 1e-14 * g["dt0"][0]
    for k in range(30):
        o.steps(1)
        f, r = o.array("fint"), g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert np.linalg.norm(f - r) <= 1e-12 * np.linalg.norm(r), k
    x = o.array("coords")
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-12 * np.max(np.abs(g["final_coords"]))


def test_steps_hex_pulse_two_materials():
    """The two bonded materials on a hex8 bar with the Pulse time step: the power iteration's
    element stiffness takes each element's own Hooke matrix (Element3D.C:242-333 reads the
    element's material); lumped mass bitwise, 30 steps to rounding (K.x summed in element order),
    the tabular target past yield."""
    g = golden("steps_two_hex.npz")
    o = Oracle(meshes.impact_two_materials_hex(4, 12))
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert abs(o.get("dt") - g["dt0"][0]) <= 1e-14 * g["dt0"][0]
    for k in range(30):
        o.steps(1)
        f, r = o.array("fint"), g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert np.linalg.norm(f - r) <= 1e-12 * np.linalg.norm(r), k
    x = o.array("coords")
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-12 * np.max(np.abs(g["final_coords"]))
    assert g["final_evp"].max() > 1e-3


def test_imposed_speed_steps_and_run_vs_reference():
    """The tensile bar with BoundarySpeed::applyConstant on its pulled end (Boundary.C:478-525:
    a = 0, v = the imposed speed and delta_disp = v dt on both nodal fields) and BoundaryRestrain
    1 1 1 on the other: lumped mass bitwise, 30 Pulse steps (K x summed in element order, so to
    rounding), then a full run pulled at 5 m/s to 2 ms (373 increments, plastic) vs the reference."""
    g = golden("steps_speed.npz")
    m = meshes.necking_bar(4, 12)
    o = Oracle(m)
    o.prologue()
    assert np.array_equal(o.array("Mass"), g["mass"])
    assert abs(o.get("dt") - g["dt0"][0]) <= 1e-14 * g["dt0"][0]
    for k in range(30):
        o.steps(1)
        f, r = o.array("fint"), g["fint"][k]
        if np.linalg.norm(r) > 0:
            assert np.linalg.norm(f - r) <= 1e-11 * np.linalg.norm(r), k
    x = o.array("coords")
    assert np.max(np.abs(x - g["final_coords"])) <= 1e-12 * np.max(np.abs(g["final_coords"]))
    top = m.bcs[1].nodes
    assert np.array_equal(o.array("v").reshape(-1, 3)[top, 2], np.full(top.size, 1.0))
    assert np.array_equal(g["final_v"].reshape(-1, 3)[top, 2], np.full(top.size, 1.0))
    r = golden("run_speed.npz")
    o = Oracle(meshes.necking_bar(4, 12, speed=5.0, tend=2e-3))
    o.prologue()
    total = 0
    while True:
        k = o.steps(100)
        total += k
        if k < 100:
            break
    assert total == int(r["increments"][0])
    x = o.array("coords")
    assert np.max(np.abs(x - r["final_coords"])) <= 1e-12 * np.max(np.abs(r["final_coords"]))
    assert np.max(np.abs(o.array("evp") - r["final_evp"])) <= 1e-12 * np.max(r["final_evp"])
    assert r["final_evp"].max() > 0.1  # the run is plastic


# ---------------------------------------------------------------------- known answers
def test_chung_hulbert_parameters():
    o = Oracle(meshes.taylor_axi(2, 2))
    assert abs(o.get("alphaM") - 0.350016) < 1e-6
    assert abs(o.get("beta") - 0.651521) < 1e-6
    assert abs(o.get("gamma") - 1.149984) < 1e-6
    assert abs(o.get("omegaS") - 1.981819) < 1e-6


def test_total_mass_axisymmetric():
    """sum of lumped masses = rho * integral of 2 pi r dA = rho pi R^2 L for the undeformed bar."""
    m = meshes.taylor_axi(5, 50)
    o = Oracle(m)
    o.prologue()
    total = o.array("mass").sum()
    exact = m.density * np.pi * 3.2e-3 ** 2 * 32.4e-3
    assert abs(total - exact) <= 1e-12 * exact


def test_total_mass_hex():
    m = meshes.taylor_hex(8, 4)
    o = Oracle(m)
    o.prologue()
    vol = 0.0
    x = m.coords[m.conn]
    for e in range(m.E):
        ext = x[e].max(axis=0) - x[e].min(axis=0)
        vol += np.prod(ext)
    assert abs(o.array("mass").sum() - m.density * vol) <= 1e-10 * m.density * vol


def _single_element(F_disp, etype=0):
    """One element, zero state, Current delta_disp = F_disp applied to the nodes."""
    m = meshes.taylor_axi(1, 1) if etype == 0 else meshes.taylor_hex(1, 1)
    m.bcs = []
    o = Oracle(m)
    x = m.coords.copy()
    x[:, 0] += 1e-3  # keep the axisymmetric element off the axis
    du = np.zeros((m.N, 3))
    du[:, :m.dim] = F_disp(x)[:, :m.dim]
    o.inject(coords=x, du=du, v=np.zeros_like(du), a=np.zeros_like(du), disp=np.zeros_like(du),
             S=np.zeros((m.E, m.nip, 3, 3)), Eps=np.zeros((m.E, m.nip, 3, 3)),
             EpsPlas=np.zeros((m.E, m.nip, 3, 3)), p=np.zeros((m.E, m.nip)),
             evp=np.full((m.E, m.nip), 1e-10), dt=1e-8)
    o.internal_matrices()
    o.internal_forces()
    return o, m


def test_zero_increment_gives_zero_strain_identity_rotation():
    o, m = _single_element(lambda x: np.zeros_like(x), etype=1)
    assert np.all(o.array("dEps") == 0.0)
    R = o.array("R").reshape(-1, 3, 3)
    assert np.all(R == np.eye(3))


def test_rigid_rotation_gives_no_strain():
    """delta_u = (Q - I) x: F = Q, so ln U = 0 and R = Q (3D hex)."""
    th = 0.3
    Q = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1.0]])
    o, m = _single_element(lambda x: x @ (Q - np.eye(3)).T, etype=1)
    assert np.max(np.abs(o.array("dEps"))) < 1e-12
    R = o.array("R").reshape(-1, 3, 3)
    assert np.max(np.abs(R - Q)) < 1e-12


def test_uniaxial_elastic_increment_is_hooke():
    """A small uniaxial stretch in z (hex): S = 2G dev(eps), p = K tr(eps), with eps = ln(1+e)."""
    e = 1e-5
    o, m = _single_element(lambda x: np.stack([0 * x[:, 0], 0 * x[:, 1], e * x[:, 2]], 1), etype=1)
    E, nu = m.young, m.poisson
    G, K = E / (2 * (1 + nu)), E / (3 * (1 - 2 * nu))
    eps = np.log1p(e)
    S = o.array("S").reshape(-1, 3, 3)
    p = o.array("p")
    assert np.allclose(S[:, 2, 2], 2 * G * (eps - eps / 3), rtol=1e-9)
    assert np.allclose(S[:, 0, 0], 2 * G * (-eps / 3), rtol=1e-9)
    assert np.allclose(p, K * eps, rtol=1e-9)


def test_plastic_step_returns_to_yield_surface():
    """After a plastic correction the J2 stress equals sigma_y(evp) within the Newton tolerance."""
    e = 2e-2
    o, m = _single_element(lambda x: np.stack([0 * x[:, 0], 0 * x[:, 1], e * x[:, 2]], 1), etype=1)
    S = o.array("S").reshape(-1, 3, 3)
    evp = o.array("evp")
    j2 = np.sqrt(1.5 * np.sum(S * S, axis=(1, 2)))
    sy = m.A + m.B * evp ** m.n
    assert np.all(evp > 1e-10)
    assert np.all(np.abs(j2 - sy) <= 1e-8 * sy)


@pytest.mark.parametrize("name,model", [("steps_two.npz", lambda: meshes.impact_two_materials(5, 50)),
                                        ("steps_metafor.npz", lambda: meshes.metafor_bar(5, 50))])
def test_oracle_hardening_laws_and_materials_vs_reference(name, model):
    """Tabular and Metafor hardening, a material without hardening, two materials in one mesh and
    per-node initial velocities: the oracle is bit-exact with the compiled reference over 40
    steps (forces of every step, lumped mass, final coordinates)."""
    g = golden(name)
    m = model()
    o = Oracle(m)
    o.prologue()
    assert np.array_equal(o.array("mass"), g["mass"][::2])
    for k in range(40):
        assert o.steps(1) == 1
        assert np.array_equal(o.array("fint"), g["fint"][k]), k
    assert np.array_equal(o.array("coords"), g["final_coords"])
    assert np.array_equal(o.array("evp"), g["final_evp"])
    assert g["final_evp"].max() > 0  # the laws were exercised past yield
