"""The 3D Taylor bar at the benchmark's size (40x40 cross-section grid clipped to the radius, 400
layers: 505,600 ElHex8n3D, 539,345 nodes, Pulse time step) against the oracle on the same mesh.

The oracle cannot run the whole 80 us here, so the bar is compared where a CPU can follow it: the
prologue and first steps from t = 0 (1e-12 on the forces, as on the small bars), and one element
pass from the GPU's own mid-run state at t = 10 us -- the window bench.py times, with the impact
end plastic -- injected into the oracle (1e-12 on the forces and on the updated state).  Runs are
deterministic: the CSR assembly has no atomics, so two handles give the same trajectory bit for
bit.  The two gradient workloads at their sizes -- the 20x200 axisymmetric bar and the 209,824-element
necking bar through the batched path -- are held to the sensitivity oracle over their first steps."""

import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
STATE_TOL = 1e-12


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def bar():
    m = meshes.taylor_hex(40, 400)
    assert m.E == 505600
    return m


def test_full_size_prologue_and_first_steps_vs_oracle(gpu_lib, bar):
    o = Oracle(bar, threads=os.cpu_count() or 1)
    o.prologue()
    d = gpu_lib.GpuDomain(bar)
    d.prologue()
    assert rel(d.get_state("mass")["mass"], o.array("mass")) == 0.0
    assert abs(d.time_step() - o.get("dt")) <= 1e-10 * o.get("dt")
    for k in range(3):
        o.steps(1)
        assert d.step(1) == 1
        fo = o.array("fint")
        if np.linalg.norm(fo) > 0:
            assert rel(d.fint(), fo) <= FORCE_TOL, k
        assert abs(d.time_info()["time"] - o.get("time")) <= 1e-10 * o.get("time")
    x, xo = d.get_state("coords")["coords"].ravel(), o.array("coords")
    assert np.max(np.abs(x - xo)) <= 1e-12 * np.max(np.abs(xo))


def test_full_size_mid_run_pass_vs_oracle(gpu_lib, bar):
    d = gpu_lib.GpuDomain(bar)
    d.prologue()
    while d.time_info()["time"] < 10e-6:
        assert d.step(50) > 0
    info = d.time_info()
    st = d.get_state("coords", "du", "v", "a", "disp", "S", "Eps", "EpsPlas", "p", "evp")
    assert np.max(st["evp"]) > 1e-3  # the impact end has yielded
    o = Oracle(bar, threads=os.cpu_count() or 1)
    o.prologue()
    o.inject(coords=st["coords"], du=st["du"], v=st["v"], a=st["a"], disp=st["disp"], S=st["S"],
             Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"], dt=info["time_step"])
    o.internal_matrices()
    fo = o.internal_forces()
    f = d.internal_forces(coords=st["coords"], du=st["du"], dt=info["time_step"])
    assert rel(f, fo) <= FORCE_TOL
    out = d.get_state("S", "EpsPlas", "evp", "p")
    for k in out:
        assert rel(out[k], o.array(k)) <= STATE_TOL, k


def test_full_size_runs_are_deterministic(gpu_lib, bar):
    runs = []
    for _ in range(2):
        d = gpu_lib.GpuDomain(bar)
        d.prologue()
        assert d.step(30) == 30
        runs.append((d.get_state("coords")["coords"], d.fint()))
        d.close()
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def _rel_p(dx, dxo, p):
    return np.linalg.norm(dx[p] - dxo[p]) / np.linalg.norm(dxo[p])


def test_full_size_gradient_bar_vs_dual_oracle(gpu_lib):
    """The gradient workload's bar (20x200 ElQua4nAx, 4,000 elements), the first 200 steps of its
    Courant schedule: derivatives of the final coordinates w.r.t. A, B, n, |v0| vs the sensitivity
    oracle (FP64 dual numbers) to 1e-5, coordinates to 1e-12."""
    from oracle.oracle import SensOracle
    m = meshes.taylor_axi(20, 200)
    o = Oracle(m)
    o.prologue()
    mass = o.array("mass").copy()
    dts = []
    for _ in range(200):
        dts.append(o.get("dt"))
        o.steps(1)
    dts = np.array(dts)
    s = SensOracle(m, mass=mass, threads=os.cpu_count() or 1)
    s.run(dts)
    xo, dxo = s.coords()
    x, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    assert np.max(np.abs(x - xo)) <= 1e-12 * np.max(np.abs(xo))
    for p in range(4):
        assert np.linalg.norm(dxo[p]) > 0, p
        assert _rel_p(dx, dxo, p) <= 1e-5, (p, _rel_p(dx, dxo, p))


def test_full_size_necking_batch_vs_dual_oracle(gpu_lib):
    """The batched gradient workload's bar (209,824 hex8 necking bar, mass scaling x100), two
    parameter sets through dnl_batch_sens_run over the first steps of its 3.55e-7 s schedule: the
    first instance's derivatives vs the sensitivity oracle on the same bar to 1e-5 (the parameters
    whose derivative is not yet zero), the second instance equal to its own single-mesh run."""
    from oracle.oracle import SensOracle
    models = meshes.necking_batch(2, seed=0, nz=166)
    assert models[0].E == 209824
    dts = np.full(2, models[0].tend / 30000)
    out = gpu_lib.BatchDomain(models).sensitivities(dts)
    g = gpu_lib.GpuDomain(models[0])
    g.prologue()
    mass = g.get_state("mass")["mass"].ravel().copy()
    g.close()
    s = SensOracle(models[0], mass=mass, threads=os.cpu_count() or 1)
    s.run(dts)
    xo, dxo = s.coords()
    x, dx = out[0]
    assert np.max(np.abs(x - xo)) <= 1e-12 * np.max(np.abs(xo))
    checked = 0
    for p in range(4):
        if np.linalg.norm(dxo[p]) == 0:
            assert not np.any(dx[p]), p
            continue
        assert _rel_p(dx, dxo, p) <= 1e-5, (p, _rel_p(dx, dxo, p))
        checked += 1
    assert checked >= 1
    x1, dx1 = gpu_lib.GpuDomain(models[1]).sensitivities(dts)
    assert np.array_equal(out[1][0], x1) and np.array_equal(out[1][1], dx1)


def _gradient_workload(gpu_lib):
    """The gradient configuration: the 20x200 axisymmetric bar, the schedule of the nominal run's
    own Courant steps (4,000), the target shape of (A, B, n) = (110 MPa, 310 MPa, 0.28) and
    L = mean over the free-surface nodes of |x_final - x_target|^2."""
    m = meshes.taylor_axi(20, 200)
    v0 = float(np.linalg.norm(m.v0))
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    dts = []
    while len(dts) < 4000:
        dts.append(d.time_info()["time_step"])
        assert d.step(1) == 1
    d.close()
    dts = np.array(dts)
    target = gpu_lib.model_with_params(m, 110e6, 310e6, 0.28, v0)
    xt, _ = gpu_lib.GpuDomain(target).sensitivities(dts)
    surf = meshes.taylor_axi_free_surface(20, 200)
    return m, v0, dts, xt, surf


def test_full_size_gradient_vs_central_differences(gpu_lib):
    """The gradient configuration's dL/d(A, B, n, |v0|) against central differences of L computed
    by the same GPU run, h = 1e-5 relative per parameter: within 1e-5 relative for all four.

    The difference quotient carries the rounding noise of L (a small mismatch of two 4,000-step
    shapes, with elastic/plastic switches inside [p - h, p + h]) divided by 2h, so its distance from
    the derivative does not shrink with h below ~1e-5: a sweep of h from 1e-2 to 1e-7 measured the
    quotient for n 2.2e-6 away at 1e-5, 2.7e-5 at 1e-6 and 5.9e-6 at 1e-7, and a four-point stencil
    no closer (3.2e-5 at 1e-6); the least distance, over all four parameters, lies at h = 3e-5 to
    3e-4 relative (<= 1.1e-6)."""
    m, v0, dts, xt, surf = _gradient_workload(gpu_lib)
    d = gpu_lib.GpuDomain(m)
    x, dx = d.sensitivities(dts)
    w = np.zeros((m.N, 3))
    w[surf] = 2.0 * (x[surf] - xt[surf]) / len(surf)
    g = np.einsum("pnj,nj->p", dx, w)
    pv = np.array([m.A, m.B, m.n, v0])

    def loss(q):
        d.reset(gpu_lib.model_with_params(m, *q))
        xq, _ = d.sensitivities(dts)
        return float(np.mean(np.sum((xq[surf] - xt[surf]) ** 2, axis=1)))

    for p in range(4):
        h = 1e-5 * pv[p]
        e = np.eye(4)[p]
        fd = (loss(pv + h * e) - loss(pv - h * e)) / (2 * h)
        err = abs(fd - g[p]) / abs(g[p])
        assert err <= 1e-5, (p, err, fd, g[p])


def test_full_size_gradient_reverse_mode(gpu_lib):
    """The gradient configuration in reverse mode: dnl_adjoint_forward / dnl_adjoint_backward with
    ceil(sqrt(4000)) = 64 steps per checkpoint equal the forward-mode gradient to 1e-10 per
    parameter; 63 checkpoints and one segment of step states held, every step run twice."""
    m, v0, dts, xt, surf = _gradient_workload(gpu_lib)
    d = gpu_lib.GpuDomain(m)
    x, dx = d.sensitivities(dts)
    w = np.zeros((m.N, 3))
    w[surf] = 2.0 * (x[surf] - xt[surf]) / len(surf)
    g_fwd = np.einsum("pnj,nj->p", dx, w)
    d.reset()
    g_rev = d.adjoint(w, dts, 0)
    st = d.adjoint_stats()
    assert st["stride"] == 64 and st["checkpoints"] == 63 and st["recomputed_steps"] == 4000
    for p in range(4):
        err = abs(g_rev[p] - g_fwd[p]) / abs(g_fwd[p])
        assert err <= 1e-10, (p, err, g_rev[p], g_fwd[p])
