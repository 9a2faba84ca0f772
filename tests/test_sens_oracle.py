"""The sensitivity oracle (oracle/dnl_sens.cc): FP64 dual numbers through the restated explicit run.

* its value part repeats the primal oracle's arithmetic: same final coordinates, bit for bit, for
  the same step-size schedule;
* its tangents agree with central finite differences of the run (h = 1e-6 relative, the
  difference step of the gradient checks): axisymmetric to 1e-5; in 3D the finite differences
  themselves carry ~1e-9 relative noise from the Jacobi pivot choice on the bar's symmetry planes,
  so h = 1e-5 and a 1e-3 tolerance there.  The one-point hexahedron's coarse bar has small
  derivatives (~1e-12 m/Pa for A) under the same noise: the distance to the difference quotient
  falls as 1/h down to 2e-5 at h = 1e-3 (1.4e-3 at 1e-5, 1.5e-2 at 1e-6), so h = 1e-3 and 1e-4.
"""

import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle, SensOracle
from redynela_gb300 import meshes


def schedule(m, nsteps):
    o = Oracle(m)
    o.prologue()
    dts = []
    for _ in range(nsteps):
        dts.append(o.get("dt"))
        o.steps(1)
    return np.array(dts), o.array("coords").reshape(-1, 3).copy(), o.array("mass").copy()


def perturbed(m, p, h):
    if p == 3:
        return dataclasses.replace(m, v0=tuple(np.asarray(m.v0) * (1 + h)))
    name = "ABn"[p]
    return dataclasses.replace(m, **{name: getattr(m, name) * (1 + h)})


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def model(kind):
    return {"axi": lambda: meshes.taylor_axi(5, 30), "hex": lambda: meshes.taylor_hex(3, 6),
            "tet4": lambda: meshes.taylor_tet(4, 6), "tet10": lambda: meshes.taylor_tet(3, 4, quadratic=True),
            "hex1pt": lambda: meshes.taylor_hex_1pt(4, 8)}[kind]()


# ElTet10n3D: two steps (the reference's element blows up after them: negative lumped corner masses)
@pytest.mark.parametrize("etype,nsteps", [("axi", 60), ("hex", 60), ("tet4", 60), ("tet10", 2),
                                          ("hex1pt", 60)])
def test_value_part_is_the_primal_oracle(etype, nsteps):
    m = model(etype)
    dts, x_ref, mass = schedule(m, nsteps)
    s = SensOracle(m, mass=mass)
    s.run(dts)
    x, dx = s.coords()
    assert np.array_equal(x, x_ref)
    assert np.all(np.isfinite(dx))


@pytest.mark.parametrize("etype,nsteps,h,tol", [("axi", 150, 1e-6, 1e-5), ("hex", 60, 1e-5, 1e-3),
                                                ("tet4", 60, 1e-5, 1e-3), ("tet10", 1, 1e-5, 1e-3),
                                                ("hex1pt", 60, 1e-3, 1e-4)])
def test_tangents_vs_central_differences(etype, nsteps, h, tol):
    m = {"axi": lambda: meshes.taylor_axi(4, 30), "hex": lambda: meshes.taylor_hex(3, 8)}.get(
        etype, lambda: model(etype))()
    dts, _, mass = schedule(m, nsteps)
    s = SensOracle(m, mass=mass)
    s.run(dts)
    _, dx = s.coords()
    for p in range(4):
        val = [m.A, m.B, m.n, float(np.linalg.norm(m.v0))][p]
        xs = []
        for sign in (1, -1):
            o = SensOracle(perturbed(m, p, sign * h), mass=mass)
            o.run(dts)
            xs.append(o.coords()[0])
        fd = (xs[0] - xs[1]) / (2 * h * val)
        if etype == "tet10" and p < 3:  # one step, every point elastic: the hardening plays no part
            assert not np.any(dx[p]) and not np.any(fd), p
            continue
        assert np.linalg.norm(dx[p]) > 0, p
        assert rel(dx[p], fd) <= tol, (p, rel(dx[p], fd))
