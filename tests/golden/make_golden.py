"""Regenerate the golden fixtures of tests/golden from the compiled reference.

Needs the reference DynELA numerical core built by ``make -C oracle ref`` (it compiles the
reference sources where they lie; only possible where those sources exist).  Every fixture is the
reference's own output on a seeded synthetic model:

* ``tables.npz``        element tables of ElQua4nAx / ElHex8n3D / ElQua4n2D
* ``forces_axi.npz``    one Domain::computeInternalForces on an injected mid-run state, 3x4 axi bar
* ``forces_hex.npz``    the same on a 4x4x3 hex bar
* ``steps_c0.npz``      the 5x50 Taylor bar, first 20 steps: Fint, dt, kinetic energy per step
* ``run_c0.npz``        the 5x50 Taylor bar to 80 us: final coordinates, plastic strain, pressure
* ``steps_hex.npz``     a 6x6x8 hex bar with the Pulse time step, first 30 steps
* ``run_hex.npz``       an 8x8x24 hex bar with the Pulse time step to 80 us: final coordinates
* ``steps_two.npz``     two bonded materials in the pattern of Samples/Traction (tabular target,
                        elastic projectile with its own initial velocity), first 40 steps
* ``steps_metafor.npz`` the 5x50 bar with an IsoHardMetafor law, first 40 steps
* ``steps_two_hex.npz`` the same two bonded materials on a 4x4x12-cell ElHex8n3D bar with the Pulse
                        time step (each element's own Hooke matrix in the power iteration), first 30
                        steps
* ``results_axi.bin``   the reference's binary results file (Structure::writeData) of the 3x4 axi bar
                        after 13 steps, and ``results_axi.npz`` its state from the harness
* ``forces_plane.npz``  one Domain::computeInternalForces on an injected state, 3x4 ElQua4n2D bar
* ``steps_plane.npz``   the 5x50 bar in plane strain (ElQua4n2D), first 40 steps
* ``run_plane.npz``     the same bar to 80 us: final coordinates, plastic strain, pressure
* ``steps_plane_pulse.npz`` the plane-strain bar with the Pulse time step, first 30 steps
* ``forces_tet4.npz``, ``forces_tet10.npz``  one computeInternalForces on an injected state of a
                        4x4x3-cell bar split into ElTet4n3D / ElTet10n3D
* ``steps_tet4.npz``    the 6x6x8-cell ElTet4n3D bar (Courant, safety 0.5), first 40 steps
* ``run_tet4.npz``      the same bar to 80 us
* ``steps_tet4_pulse.npz`` the same bar with the Pulse time step, first 20 steps
* ``steps_tet10.npz``   the ElTet10n3D bar, lumped mass and its first 2 steps (the reference's run
                        of this element ends in a singular Jacobian a few steps later)
* ``steps_speed.npz``   a coarse tensile bar of ElHex8n3D (necking_bar(4, 12): one end clamped by
                        BoundaryRestrain 1 1 1, the other pulled by BoundarySpeed 0 0 1 m/s), Pulse
                        time step, lumped mass and its first 30 steps
* ``run_speed.npz``     the same bar pulled at 5 m/s to 2 ms: final coordinates, velocities, plastic
                        strain
* ``forces_mixed.npz``  one computeInternalForces on an injected state of a 4x4x3-cell bar of
                        ElTet4n3D (first layer) and ElHex8n3D (the others) in one domain
* ``steps_mixed.npz``   the 6x6x12-cell bar of ElTet4n3D (6 layers) and ElTet10n3D (6 layers) in one
                        domain, Courant time step: lumped mass and its first 5 steps (its ElTet10n3D
                        part ends in a singular Jacobian a few steps later, as the ElTet10n3D bar)
* ``forces_mixed_two.npz`` the force pass of ``forces_mixed.npz`` with the ElTet4n3D layer of a
                        tabular-hardening material and the ElHex8n3D layers of a power-law one
* ``steps_mixed_two.npz`` the ElTet4n3D + ElTet10n3D bar of ``steps_mixed.npz`` with the two parts
                        of two materials (other E, nu, rho and hardening above): lumped mass, time
                        steps and its first 3 steps
* ``results_mixed.bin`` the reference's results file of the 3x3x4-cell bar of ElTet4n3D (2 layers)
                        and ElTet10n3D (2 layers) after its first 2 steps (the first step's
                        element pass sees the bar at rest): each element's own integration points,
                        elements in the domain's order (its ElTet10n3D part ends in a singular
                        Jacobian at the fourth step)

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dnl_io, states  # noqa: E402
from redynela_gb300 import meshes  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path)} bytes")


def results():
    """The results-file fixture only: python tests/golden/make_golden.py results"""
    m = meshes.taylor_axi(3, 4)
    path = os.path.join(HERE, "results_axi.bin")
    r = dnl_io.run_reference("steps", m, 13, path)
    print(f"results_axi.bin: {os.path.getsize(path)} bytes")
    save("results_axi.npz", **{k: r[k] for k in r if k.startswith("final_")}, time=r["time"])
    results_mixed()


def results_mixed():
    """The mixed-domain results file only: python tests/golden/make_golden.py results_mixed"""
    m = meshes.taylor_mixed(3, 4, nz_lower=2)
    path = os.path.join(HERE, "results_mixed.bin")
    dnl_io.run_reference("steps", m, 2, path)
    print(f"results_mixed.bin: {os.path.getsize(path)} bytes")


def laws():
    """The hardening-law / material fixtures only: python tests/golden/make_golden.py laws"""
    for name, m in (("steps_two.npz", meshes.impact_two_materials(5, 50)),
                    ("steps_metafor.npz", meshes.metafor_bar(5, 50))):
        r = dnl_io.run_reference("steps", m, 40)
        save(name, mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
             fint=np.stack([r[f"fint_{k:06d}"] for k in range(40)]),
             final_coords=r["final_coords"], final_evp=r["final_evp"], final_S=r["final_S"],
             final_p=r["final_p"])


def laws3d():
    """The 3D two-material fixture only: python tests/golden/make_golden.py laws3d"""
    m = meshes.impact_two_materials_hex(4, 12)
    r = dnl_io.run_reference("steps", m, 30)
    save("steps_two_hex.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         fint=np.stack([r[f"fint_{k:06d}"] for k in range(30)]), final_coords=r["final_coords"],
         final_evp=r["final_evp"], final_S=r["final_S"])


def plane():
    """The plane-strain (ElQua4n2D) fixtures only: python tests/golden/make_golden.py plane"""
    save("tables.npz", **dnl_io.reference_tables())
    m = meshes.taylor_plane(3, 4)
    st = states.random_state(m, seed=7)
    r = dnl_io.run_reference("forces", m, state=st)
    save("forces_plane.npz", **{f"in_{k}": np.asarray(v) for k, v in st.items()}, fint=r["fint"],
         **{k: r[k] for k in r if k.startswith("out_")})
    m = meshes.taylor_plane(5, 50)
    r = dnl_io.run_reference("steps", m, 40)
    save("steps_plane.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(40)]),
         final_coords=r["final_coords"], final_evp=r["final_evp"], final_S=r["final_S"],
         final_p=r["final_p"])
    mp = dataclasses.replace(m, method=meshes.PULSE)
    r = dnl_io.run_reference("steps", mp, 30)
    save("steps_plane_pulse.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(30)]),
         final_coords=r["final_coords"])
    r = dnl_io.run_reference("run", m)
    save("run_plane.npz", increments=r["increments"], time=r["time"],
         final_coords=r["final_coords"], final_evp=r["final_evp"], final_p=r["final_p"],
         final_S=r["final_S"], final_v=r["final_v"])


def tets():
    """The tetrahedron fixtures only: python tests/golden/make_golden.py tets"""
    save("tables.npz", **dnl_io.reference_tables())
    for name, q in (("forces_tet4.npz", False), ("forces_tet10.npz", True)):
        m = meshes.taylor_tet(4, 3, quadratic=q)
        st = states.random_state(m, seed=7)
        r = dnl_io.run_reference("forces", m, state=st)
        save(name, **{f"in_{k}": np.asarray(v) for k, v in st.items()}, fint=r["fint"],
             **{k: r[k] for k in r if k.startswith("out_")})
    m = meshes.taylor_tet(6, 8)
    r = dnl_io.run_reference("steps", m, 40)
    save("steps_tet4.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(40)]),
         final_coords=r["final_coords"], final_S=r["final_S"])
    r = dnl_io.run_reference("steps", dataclasses.replace(m, method=meshes.PULSE), 20)
    save("steps_tet4_pulse.npz", dt0=r["dt0"], dt=r["dt"],
         fint=np.stack([r[f"fint_{k:06d}"] for k in range(20)]), final_coords=r["final_coords"])
    r = dnl_io.run_reference("run", m)
    save("run_tet4.npz", increments=r["increments"], time=r["time"],
         final_coords=r["final_coords"], final_evp=r["final_evp"], final_p=r["final_p"])
    m = meshes.taylor_tet(6, 8, quadratic=True)
    r = dnl_io.run_reference("steps", m, 2)
    save("steps_tet10.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(2)]),
         final_coords=r["final_coords"])


def speed():
    """The imposed-velocity (BoundarySpeed) fixtures only: python tests/golden/make_golden.py speed"""
    m = meshes.necking_bar(4, 12)
    r = dnl_io.run_reference("steps", m, 30)
    save("steps_speed.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(30)]),
         final_coords=r["final_coords"], final_v=r["final_v"], final_S=r["final_S"])
    m = meshes.necking_bar(4, 12, speed=5.0, tend=2e-3)
    r = dnl_io.run_reference("run", m)
    save("run_speed.npz", increments=r["increments"], time=r["time"],
         final_coords=r["final_coords"], final_v=r["final_v"], final_evp=r["final_evp"])


def mixed():
    """The mixed element-type fixtures only: python tests/golden/make_golden.py mixed

    Only what the reference computes soundly: a hexahedron + tetrahedron domain is pinned by one
    force pass (elements created tetrahedra first; the reverse order, and its Pulse loop, make
    Vector::redim copy a longer vector into a shorter one, a heap overflow), and the time steps by
    the ElTet4n3D + ElTet10n3D domain with the Courant step."""
    m = meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D, upper=meshes.ELHEX8N3D)
    st = states.random_state(m, seed=7)
    r = dnl_io.run_reference("forces", m, state=st)
    save("forces_mixed.npz", **{f"in_{k}": np.asarray(v) for k, v in st.items()}, fint=r["fint"],
         **{k: r[k] for k in r if k.startswith("out_")})
    m = meshes.taylor_mixed(6, 12)
    r = dnl_io.run_reference("steps", m, 5)
    save("steps_mixed.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(5)]),
         final_coords=r["final_coords"], final_S=r["final_S"], final_p=r["final_p"])


def mixed_materials():
    """The mixed element-type, two-material fixtures only:
    python tests/golden/make_golden.py mixed_materials"""
    tx, ty = meshes.tabular_table(360e6, 316e6, 0.28)
    target = meshes.MaterialLaw(74.2e9, 0.33, 2784.0, meshes.HARD_TABULAR, (), tx, ty)
    copper = meshes.MaterialLaw(117e9, 0.35, 8930.0, meshes.HARD_POWER, (90e6, 292e6, 0.31))
    m = meshes.group_materials(meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D,
                                                   upper=meshes.ELHEX8N3D), [target, copper])
    st = states.random_state(m, seed=7)
    r = dnl_io.run_reference("forces", m, state=st)
    save("forces_mixed_two.npz", **{f"in_{k}": np.asarray(v) for k, v in st.items()}, fint=r["fint"],
         **{k: r[k] for k in r if k.startswith("out_")})
    steel = meshes.MaterialLaw(193.6e9, 0.3, 7800.0, meshes.HARD_POWER, (250e6, 400e6, 0.4))
    m = meshes.group_materials(meshes.taylor_mixed(6, 12), [copper, steel])
    r = dnl_io.run_reference("steps", m, 3)
    save("steps_mixed_two.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         fint=np.stack([r[f"fint_{k:06d}"] for k in range(3)]), final_coords=r["final_coords"],
         final_S=r["final_S"])


def main():
    if not dnl_io.reference_available():
        sys.exit("compiled reference missing: run `make -C oracle ref`")
    if sys.argv[1:] == ["results"]:
        results()
        return
    if sys.argv[1:] == ["results_mixed"]:
        results_mixed()
        return
    if sys.argv[1:] == ["laws"]:
        laws()
        return
    if sys.argv[1:] == ["plane"]:
        plane()
        return
    if sys.argv[1:] == ["laws3d"]:
        laws3d()
        return
    if sys.argv[1:] == ["tets"]:
        tets()
        return
    if sys.argv[1:] == ["speed"]:
        speed()
        return
    if sys.argv[1:] == ["mixed"]:
        mixed()
        return
    if sys.argv[1:] == ["mixed_materials"]:
        mixed_materials()
        return
    t = dnl_io.reference_tables()
    save("tables.npz", **t)

    for name, m in (("forces_axi.npz", meshes.taylor_axi(3, 4)),
                    ("forces_hex.npz", meshes.taylor_hex(4, 3))):
        st = states.random_state(m, seed=7)
        r = dnl_io.run_reference("forces", m, state=st)
        save(name, **{f"in_{k}": np.asarray(v) for k, v in st.items()}, fint=r["fint"],
             **{k: r[k] for k in r if k.startswith("out_")})

    m = meshes.taylor_axi(5, 50)
    r = dnl_io.run_reference("steps", m, 20)
    save("steps_c0.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(20)]),
         final_coords=r["final_coords"], final_evp=r["final_evp"], final_p=r["final_p"])

    r = dnl_io.run_reference("run", m)
    save("run_c0.npz", increments=r["increments"], time=r["time"], final_coords=r["final_coords"],
         final_evp=r["final_evp"], final_p=r["final_p"], final_S=r["final_S"],
         final_v=r["final_v"])

    m = meshes.taylor_hex(6, 8)
    r = dnl_io.run_reference("steps", m, 30)
    save("steps_hex.npz", mass=r["mass"], dt0=r["dt0"], dt=r["dt"], time=r["time"],
         kinetic=r["kinetic"], fint=np.stack([r[f"fint_{k:06d}"] for k in range(30)]),
         final_coords=r["final_coords"])

    m = meshes.taylor_hex(8, 24)
    r = dnl_io.run_reference("run", m)
    save("run_hex.npz", increments=r["increments"], time=r["time"], final_coords=r["final_coords"],
         final_evp=r["final_evp"])

    results()
    laws()
    laws3d()
    plane()
    tets()
    speed()
    mixed()
    mixed_materials()


if __name__ == "__main__":
    main()
