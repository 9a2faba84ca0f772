"""The sensitivity oracle (oracle/dnl_sens.cc): FP64 dual numbers through the restated explicit run.

* its value part repeats the primal oracle's arithmetic: same final coordinates, bit for bit, for
  the same step-size schedule;
* its tangents agree with central finite differences of the run (h = 1e-6 relative, the
  difference step of the gradient checks): axisymmetric to 1e-5; in 3D the finite differences
  themselves carry ~1e-9 relative noise from the Jacobi pivot choice on the bar's symmetry planes,
  so h = 1e-5 and a 1e-3 tolerance there.
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


@pytest.mark.parametrize("etype", ["axi", "hex"])
def test_value_part_is_the_primal_oracle(etype):
    m = meshes.taylor_axi(5, 30) if etype == "axi" else meshes.taylor_hex(3, 6)
    dts, x_ref, mass = schedule(m, 60)
    s = SensOracle(m, mass=mass)
    s.run(dts)
    x, dx = s.coords()
    assert np.array_equal(x, x_ref)
    assert np.all(np.isfinite(dx))


@pytest.mark.parametrize("etype,nsteps,h,tol", [("axi", 150, 1e-6, 1e-5), ("hex", 60, 1e-5, 1e-3)])
def test_tangents_vs_central_differences(etype, nsteps, h, tol):
    m = meshes.taylor_axi(4, 30) if etype == "axi" else meshes.taylor_hex(3, 8)
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
        assert np.linalg.norm(dx[p]) > 0, p
        assert rel(dx[p], fd) <= tol, (p, rel(dx[p], fd))
