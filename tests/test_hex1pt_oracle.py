"""The one-point hexahedron with viscous hourglass control (DNL_ELHEX8N3D_1PT, not a reference
element: the reference integrates ElHex8n3D at 2x2x2 points and has no hourglass control) on the
oracle, which restates its formulation: properties of the hourglass forces, the lumped mass, and a
full Taylor run.  CPU only."""

import numpy as np

from oracle import states
from oracle.oracle import Oracle
from redynela_gb300 import meshes

# ElHex8n3D's node signs (bottom face counter-clockwise, then the top face)
XI = np.array([-1, 1, 1, -1, -1, 1, 1, -1])
ETA = np.array([-1, -1, 1, 1, -1, -1, 1, 1])


def _forces(m, st, v, coefficient):
    o = Oracle(m)
    o.L.dnlo_set_hourglass(o.h, coefficient)
    o.inject(**dict(st, v=v))
    o.internal_matrices()
    return o.internal_forces().reshape(-1, 3)


def test_hourglass_forces_vanish_on_linear_fields_and_resist_hourglass_modes():
    m = meshes.taylor_hex_1pt(8, 12)
    st = states.random_state(m, seed=3, du_scale=0.0)
    st["coords"] = m.coords.copy()
    x = st["coords"]
    fields = {"translation": np.tile([1.0, -2.0, 3.0], (m.N, 1)),
              "linear": x @ np.array([[0.1, 0.3, -0.2], [0.05, -0.1, 0.2], [0.3, 0.1, 0.0]]) * 1e3}
    for name, v in fields.items():
        hg = _forces(m, st, v, 0.05) - _forces(m, st, v, 0.0)
        scale = np.linalg.norm(_forces(m, st, v, 0.0))
        assert np.linalg.norm(hg) <= 1e-12 * max(scale, 1.0), name
    v = np.zeros((m.N, 3))
    v[m.conn[0], 0] = XI * ETA  # the xi-eta hourglass mode of element 0, along x
    hg = _forces(m, st, v, 0.05) - _forces(m, st, v, 0.0)
    assert np.linalg.norm(hg) > 0
    assert np.sum(hg * v) < 0  # dissipative
    # linear in the coefficient
    hg2 = _forces(m, st, v, 0.1) - _forces(m, st, v, 0.0)
    assert np.allclose(hg2, 2 * hg, rtol=1e-12, atol=1e-12 * np.abs(hg).max())


def test_lumped_mass_is_the_bar_mass():
    m = meshes.taylor_hex_1pt(8, 12)
    o = Oracle(m)
    o.prologue()
    cell = (2 * 3.2e-3 / 8) ** 2 * (32.4e-3 / 12)
    assert abs(o.array("mass").sum() - m.density * cell * m.E) <= 1e-12 * m.density * cell * m.E


def test_full_taylor_run_is_stable():
    m = meshes.taylor_hex_1pt(8, 12)
    o = Oracle(m)
    o.prologue()
    n = o.steps(10 ** 9)
    assert n > 1000 and o.get("time") >= m.tend * (1 - 1e-12)
    assert 1.5 < o.array("evp").max() < 4.0
    assert np.all(np.isfinite(o.array("coords")))
