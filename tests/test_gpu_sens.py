"""Forward-mode sensitivities on the GPU (dnl_sens_run / dnl_adjoint) against the sensitivity
oracle (FP64 dual numbers through the restated run, oracle/dnl_sens.cc), with the same step-size
schedule.  The GPU differentiates the polar decomposition with the spectral formula and the J2
return by the implicit function theorem at the converged multiplier; the oracle carries dual
numbers through the Newton iterations, which stop at a 1e-8 relative residual -- the two
derivatives agree to that order.  Tolerance on each parameter's derivative field: 1e-5 relative
(2-norm)."""

import numpy as np
import pytest

from oracle.oracle import Oracle, SensOracle
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

SENS_TOL = 1e-5


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def schedule(m, nsteps):
    o = Oracle(m)
    o.prologue()
    dts = []
    for _ in range(nsteps):
        dts.append(o.get("dt"))
        o.steps(1)
    return np.array(dts), o.array("coords").reshape(-1, 3).copy(), o.array("mass").copy()


def _model(etype):
    return {"axi": lambda: meshes.taylor_axi(5, 50), "hex": lambda: meshes.taylor_hex(4, 10),
            "tet4": lambda: meshes.taylor_tet(6, 8),
            "tet10": lambda: meshes.taylor_tet(4, 6, quadratic=True),
            "hex1pt": lambda: meshes.taylor_hex_1pt(6, 10)}[etype]()


# the tetrahedra and the one-point hexahedron: the same tangent pass, the tetrahedra's node-by-node
# kinematics and force rows, the hourglass force's tangent.  ElTet10n3D: one step -- the
# reference's element has blown up by the end of the second (negative lumped corner masses) --
# in which every point is still elastic, so only d/d|v0| is not zero and the hardening
# parameters' derivatives must be exactly zero
@pytest.mark.parametrize("etype,nsteps", [("axi", 300), ("hex", 80), ("tet4", 80), ("tet10", 1),
                                          ("hex1pt", 80)])
def test_sensitivities_vs_dual_oracle(gpu_lib, etype, nsteps):
    m = _model(etype)
    dts, x_ref, mass = schedule(m, nsteps)
    s = SensOracle(m, mass=mass)
    s.run(dts)
    xo, dxo = s.coords()
    d = gpu_lib.GpuDomain(m)
    x, dx = d.sensitivities(dts)
    pos_tol = 1e-12 if etype in ("axi", "tet10") else 1e-8
    assert np.max(np.abs(x - xo)) <= pos_tol * np.max(np.abs(xo))
    for p in range(4):
        if etype == "tet10" and p < 3:
            assert not np.any(dxo[p]) and not np.any(dx[p]), p
            continue
        assert np.linalg.norm(dxo[p]) > 0
        assert rel(dx[p], dxo[p]) <= SENS_TOL, (p, rel(dx[p], dxo[p]))


def test_sens_run_primal_is_the_plain_run(gpu_lib):
    """The primal part of dnl_sens_run, given the plain run's own step sizes, is the plain run."""
    m = meshes.taylor_axi(5, 50)
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    dts = []
    for _ in range(200):
        dts.append(d.time_info()["time_step"])
        d.step(1)
    x_plain = d.get_state("coords")["coords"]
    x, _ = gpu_lib.GpuDomain(m).sensitivities(np.array(dts))
    assert np.array_equal(x, x_plain)


REV_TOL = 1e-10  # reverse-mode vs forward-mode gradient: the same linearisation, other rounding


def _rev_vs_fwd(g, ref):
    """Largest relative difference over the parameters whose derivative is not zero; those that
    are zero (an elastic run's hardening parameters) must be zero in both."""
    worst = 0.0
    scale = np.max(np.abs(ref))
    for p in range(4):
        if ref[p] == 0.0:
            assert abs(g[p]) <= 1e-14 * scale, (p, g[p])
            continue
        worst = max(worst, abs(g[p] - ref[p]) / abs(ref[p]))
    return worst


@pytest.mark.parametrize("etype,nsteps", [("axi", 120), ("plane", 120), ("hex", 80), ("tet4", 80),
                                          ("tet10", 1), ("neck", 60)])
def test_reverse_mode_matches_forward_mode(gpu_lib, etype, nsteps):
    """dnl_adjoint (reverse sweep with checkpoints) = the forward-mode contraction (dx/dp)^T w to
    1e-10 per parameter, for a random w = dL/dx_final; plastic runs for every element type (the
    10-node tetrahedron: the one step its reference element survives, elastic), and a tensile bar
    pulled by an imposed end velocity (BoundarySpeed; starting at rest, so d/d|v0| is zero)."""
    m = {"axi": lambda: meshes.taylor_axi(4, 30), "plane": lambda: meshes.taylor_plane(4, 30),
         "hex": lambda: meshes.taylor_hex(4, 10), "tet4": lambda: meshes.taylor_tet(6, 8),
         "tet10": lambda: meshes.taylor_tet(4, 6, quadratic=True),
         "neck": lambda: meshes.necking_bar(4, 12, speed=5.0)}[etype]()
    dts, _, _ = schedule(m, nsteps)
    rng = np.random.default_rng(3)
    w = np.zeros((m.N, 3))
    w[:, :m.dim] = rng.normal(size=(m.N, m.dim))
    _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    ref = np.einsum("pnj,nj->p", dx, w)
    g = gpu_lib.GpuDomain(m).adjoint(w, dts, ckpt_stride=0)
    assert _rev_vs_fwd(g, ref) <= REV_TOL, (g, ref)
    if etype == "neck":
        assert np.all(ref[:3] != 0.0) and ref[3] == 0.0  # plastic; no initial velocity
    elif etype != "tet10":
        assert np.all(ref != 0.0)  # the run reaches the plastic range: all four derivatives live


def test_reverse_mode_checkpoint_strides(gpu_lib):
    """The gradient does not depend on the checkpoint stride (bit for bit: the recomputed steps
    are the same launches on the same states); the memory the stride sets is reported; the handle
    is back at its initial state afterwards."""
    m = meshes.taylor_axi(4, 30)
    dts, _, _ = schedule(m, 120)
    rng = np.random.default_rng(4)
    w = np.zeros((m.N, 3))
    w[:, :2] = rng.normal(size=(m.N, 2))
    d = gpu_lib.GpuDomain(m)
    grads, stats = {}, {}
    for stride in (0, 1, 7, 120):
        grads[stride] = d.adjoint(w, dts, ckpt_stride=stride)
        stats[stride] = d.adjoint_stats()
    for stride in (1, 7, 120):
        assert np.array_equal(grads[stride], grads[0]), stride
    # the default: ceil(sqrt(120)) = 11, made even so every segment replays the same graphs
    assert stats[0]["stride"] == 12 and stats[0]["checkpoints"] == 10
    assert stats[7]["checkpoints"] == 18 and stats[120]["checkpoints"] == 1
    assert stats[1]["checkpoints"] == 120 and stats[1]["recomputed_steps"] == 120
    # O(sqrt(n)) states with the default stride, against n for a stored trajectory
    assert stats[0]["checkpoint_bytes"] + stats[0]["record_bytes"] < \
        0.25 * (stats[120]["record_bytes"] + stats[1]["checkpoint_bytes"])
    x_after = d.run_schedule(dts)
    x_fresh = gpu_lib.GpuDomain(m).run_schedule(dts)
    assert np.array_equal(x_after, x_fresh)
    x_sens, _ = gpu_lib.GpuDomain(m).sensitivities(dts)
    assert np.array_equal(x_after, x_sens)  # the scheduled run is the primal of dnl_sens_run


@pytest.mark.parametrize("kind", ["axi", "hex"])
def test_reverse_mode_kept_records_equal_regenerated(gpu_lib, kind):
    """The reverse sweep keeps each segment's per-point records from its recomputation when they
    fit dnl_set_adjoint_record_budget, and otherwise runs each step's element pass again to
    regenerate them: the same records, so the same gradient bit for bit; the kept records are
    reported and the regenerating sweep holds none."""
    m = meshes.taylor_axi(4, 30) if kind == "axi" else meshes.taylor_hex(4, 10)
    dts, _, _ = schedule(m, 60)
    rng = np.random.default_rng(5)
    w = np.zeros((m.N, 3))
    w[:, :m.dim] = rng.normal(size=(m.N, m.dim))
    d = gpu_lib.GpuDomain(m)
    kept = d.adjoint(w, dts, ckpt_stride=0)
    st_kept = d.adjoint_stats()
    try:
        gpu_lib.set_adjoint_record_budget(0)
        regen = d.adjoint(w, dts, ckpt_stride=0)
        st_regen = d.adjoint_stats()
    finally:
        gpu_lib.set_adjoint_record_budget(2 << 30)
    assert np.array_equal(kept, regen)
    assert st_kept["kept_record_bytes"] > 0 and st_regen["kept_record_bytes"] == 0
    assert st_kept["bytes"] - st_regen["bytes"] == st_kept["kept_record_bytes"]


def test_torch_autograd_function(gpu_lib):
    torch = pytest.importorskip("torch")
    m = meshes.taylor_axi(4, 30)
    dts, _, _ = schedule(m, 120)
    run = gpu_lib.taylor_autograd()
    v0 = float(np.linalg.norm(m.v0))
    params = torch.tensor([m.A, m.B, m.n, v0], dtype=torch.float64, requires_grad=True)
    target = torch.from_numpy(m.coords.copy())
    x = run.apply(params, m, dts)
    loss = ((x - target) ** 2).sum()
    loss.backward()
    # the same gradient from the forward-mode derivatives, and through the forward-mode Function
    _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
    ref = np.einsum("pnj,nj->p", dx, 2 * (x.detach().numpy() - m.coords))
    assert _rev_vs_fwd(params.grad.numpy(), ref) <= REV_TOL
    pf = params.detach().clone().requires_grad_(True)
    ((gpu_lib.taylor_autograd("forward").apply(pf, m, dts) - target) ** 2).sum().backward()
    assert np.allclose(pf.grad.numpy(), ref, rtol=1e-12, atol=0)
    # and central differences of the GPU run for all four parameters (h = 1e-6 relative, 1e-5)
    for p in range(4):
        h = 1e-6 * float(params.detach()[p])
        vals = []
        for sgn in (1, -1):
            q = params.detach().clone()
            q[p] += sgn * h
            xq = run.apply(q, m, dts)
            vals.append(float(((xq - target) ** 2).sum()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - float(params.grad[p])) <= 1e-5 * abs(float(params.grad[p])), p


def test_reset_returns_to_the_initial_state(gpu_lib):
    """dnl_reset: a handle run, reset (with another material and speed) and run again gives what a
    fresh handle of that model gives, bit for bit -- plain steps and sensitivities."""
    m = meshes.taylor_axi(4, 30)
    m2 = gpu_lib.model_with_params(m, 110e6, 310e6, 0.28, 250.0)
    d = gpu_lib.GpuDomain(m)
    d.step(80)
    d.reset()
    d.step(80)
    ref = gpu_lib.GpuDomain(m)
    ref.step(80)
    assert np.array_equal(d.get_state("coords")["coords"], ref.get_state("coords")["coords"])
    d.reset(m2)
    d.step(80)
    ref2 = gpu_lib.GpuDomain(m2)
    ref2.step(80)
    assert np.array_equal(d.get_state("coords")["coords"], ref2.get_state("coords")["coords"])
    assert np.array_equal(d.get_state("S")["S"], ref2.get_state("S")["S"])
    dts, _, _ = schedule(m, 60)
    d.reset(m2)
    x, dx = d.sensitivities(dts)
    x2, dx2 = gpu_lib.GpuDomain(m2).sensitivities(dts)
    assert np.array_equal(x, x2) and np.array_equal(dx, dx2)


def _small_necking(count):
    base = meshes.necking_bar(6, 12)
    rng = np.random.default_rng(7)
    import dataclasses
    return [dataclasses.replace(base, A=float(rng.uniform(60e6, 150e6)), B=float(rng.uniform(200e6, 400e6)),
                                n=float(rng.uniform(0.2, 0.5))) for _ in range(count)]


@pytest.mark.parametrize("kind", ["hex", "axi", "tet4", "hex1pt"])
def test_batch_sensitivities_match_single_meshes(gpu_lib, kind):
    """dnl_batch_sens_run over several instances = dnl_sens_run of each instance alone, bit for
    bit (hex necking bars with three parameter sets; uneven axisymmetric, tetrahedral and one-point
    hexahedral bars)."""
    if kind in ("tet4", "hex1pt"):
        mk = meshes.taylor_tet if kind == "tet4" else meshes.taylor_hex_1pt
        models = [mk(4, 6), mk(5, 7, speed=260.0, A=120e6, n=0.45), mk(4, 5, speed=150.0, B=380e6)]
        # one schedule for all: the smallest of the instances' own stable steps
        dts = 0.8 * np.min([schedule(m, 60)[0] for m in models], axis=0)
    elif kind == "hex":
        models = _small_necking(3)
        d0 = gpu_lib.GpuDomain(models[0])
        d0.prologue()  # the Pulse estimate of the stable step
        dt0 = d0.time_step()
        dts = np.full(60, 0.5 * dt0)
    else:
        models = [meshes.taylor_axi(4, 30), meshes.taylor_axi(6, 40, speed=260.0, A=120e6, n=0.45),
                  meshes.taylor_axi(5, 20, speed=150.0, B=380e6)]
        dts, _, _ = schedule(models[0], 60)
        dts = 0.8 * dts
    b = gpu_lib.BatchDomain(models)
    out = b.sensitivities(dts)
    for i, m in enumerate(models):
        x, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
        assert np.array_equal(out[i][0], x), i
        assert np.array_equal(out[i][1], dx), i
        if kind == "hex":
            assert np.linalg.norm(dx[0]) > 0  # the pulled bar yields: dA is not zero
    b.reset()
    again = b.sensitivities(dts)
    for i in range(len(models)):
        assert np.array_equal(again[i][0], out[i][0]) and np.array_equal(again[i][1], out[i][1])


def test_hex_batch_refuses_plain_stepping(gpu_lib):
    b = gpu_lib.BatchDomain(_small_necking(2))
    with pytest.raises(gpu_lib.DnlError):
        b.step(1)


def test_graph_replay_matches_step_by_step(gpu_lib):
    """dnl_sens_run replays two-step CUDA graphs on a single mesh; a profiled run launches step by
    step.  Both, with an odd step count (the last step eager) and twice on one handle, bit for
    bit; and after dnl_reset with another material the graphs are recaptured."""
    m = meshes.taylor_axi(4, 30)
    dts, _, _ = schedule(m, 61)
    d = gpu_lib.GpuDomain(m)
    x1, dx1 = d.sensitivities(dts)
    d.reset(m)
    x2, dx2 = d.sensitivities(dts)
    ref = gpu_lib.GpuDomain(m)
    ref.profile_begin()
    x3, dx3 = ref.sensitivities(dts)
    ref.profile_end()
    for x, dx in ((x2, dx2), (x3, dx3)):
        assert np.array_equal(x, x1) and np.array_equal(dx, dx1)
    m2 = gpu_lib.model_with_params(m, 120e6, 280e6, 0.4, 240.0)
    d.reset(m2)
    x4, dx4 = d.sensitivities(dts)
    x5, dx5 = gpu_lib.GpuDomain(m2).sensitivities(dts)
    assert np.array_equal(x4, x5) and np.array_equal(dx4, dx5)
    assert not np.array_equal(x4, x1)


def test_gradient_workload_central_differences_with_tight_stopping_tests(gpu_lib):
    """The gradient workload (20x200 axisymmetric bar, its 4,000-step schedule, the squared
    distance of the free surface to the shape of (110 MPa, 310 MPa, 0.28)) at the configured
    h = 1e-6 relative: with the polar decomposition's and the radial return's stopping tests
    tightened (dnl_set_stop_tolerances 1e-15, 1e-13) the run's map is smooth at that scale and the
    central differences meet the forward-mode derivative to 1e-5 for all four parameters (measured
    2e-7 and below; with the reference's 1e-9 and 1e-8 a parameter change of 1e-6 can add or remove
    an iteration somewhere in the run and the quotient for n is 2.6e-5 away).  The default
    tolerances are restored afterwards and give the reference's results again."""
    m = meshes.taylor_axi(20, 200)
    v0 = float(np.linalg.norm(m.v0))
    d = gpu_lib.GpuDomain(m)
    d.prologue()
    dts = []
    for _ in range(4000):
        dts.append(d.time_info()["time_step"])
        d.step(1)
    dts = np.array(dts)
    surf = meshes.taylor_axi_free_surface(20, 200)
    xt = gpu_lib.GpuDomain(gpu_lib.model_with_params(m, 110e6, 310e6, 0.28, v0)).run_schedule(dts)
    pv = np.array([m.A, m.B, m.n, v0])
    x_default = gpu_lib.GpuDomain(m).run_schedule(dts)
    gpu_lib.set_stop_tolerances(1e-15, 1e-13)
    try:
        x, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
        w = np.zeros((m.N, 3))
        w[surf] = 2.0 * (x[surf] - xt[surf]) / len(surf)
        g = np.einsum("pnj,nj->p", dx, w)
        e = gpu_lib.GpuDomain(m)

        def loss(q):
            e.reset(gpu_lib.model_with_params(m, *q))
            xq = e.run_schedule(dts)
            return float(np.mean(np.sum((xq[surf] - xt[surf]) ** 2, axis=1)))

        for p in range(4):
            h = 1e-6 * pv[p]
            fd = (loss(pv + h * np.eye(4)[p]) - loss(pv - h * np.eye(4)[p])) / (2 * h)
            assert abs(fd - g[p]) <= 1e-5 * abs(g[p]), (p, fd, g[p])
    finally:
        gpu_lib.set_stop_tolerances()
    assert np.array_equal(gpu_lib.GpuDomain(m).run_schedule(dts), x_default)


@pytest.mark.parametrize("etype,nsteps", [("axi", 120), ("plane", 120), ("hex", 80), ("tet4", 80),
                                          ("hex1pt", 80), ("neck", 60), ("hex_tet", 60)])
def test_tangents_vs_central_differences_with_tight_stopping_tests(gpu_lib, etype, nsteps):
    """Every element type (and a domain of two, and the bar pulled by an imposed speed): the
    forward-mode tangents of a linear functional of the final coordinates against central
    differences of the GPU's own scheduled run at h = 1e-5 relative, with the stopping tests
    tightened (1e-15, 1e-13), to 1e-5 per parameter (measured 3.3e-7 and below).  At the
    reference's tolerances the 3D quotients carry the iterations' jumps divided by h (up to 1e-2 at
    this h on these bars), which is why the oracle's own checks of 3D tangents need h = 1e-3."""
    m = {"axi": lambda: meshes.taylor_axi(4, 30), "plane": lambda: meshes.taylor_plane(4, 30),
         "hex": lambda: meshes.taylor_hex(4, 10), "tet4": lambda: meshes.taylor_tet(6, 8),
         "hex1pt": lambda: meshes.taylor_hex_1pt(6, 10),
         "neck": lambda: meshes.necking_bar(4, 12, speed=5.0),
         "hex_tet": lambda: meshes.taylor_mixed(4, 8, lower=meshes.ELHEX8N3D,
                                                upper=meshes.ELTET4N3D)}[etype]()
    gpu_lib.set_stop_tolerances(1e-15, 1e-13)
    try:
        d = gpu_lib.GpuDomain(m)
        d.prologue()
        dts = []
        for _ in range(nsteps):
            dts.append(d.time_info()["time_step"])
            d.step(1)
        dts = np.array(dts)
        w = np.zeros((m.N, 3))
        w[:, :m.dim] = np.random.default_rng(3).normal(size=(m.N, m.dim))
        _, dx = gpu_lib.GpuDomain(m).sensitivities(dts)
        g = np.einsum("pnj,nj->p", dx, w)
        pv = np.array([m.A, m.B, m.n, np.linalg.norm(m.v0)])
        e = gpu_lib.GpuDomain(m)
        live = 0
        for p in range(4):
            if pv[p] == 0.0:  # the pulled bar starts at rest: no initial-speed derivative
                assert g[p] == 0.0
                continue
            h = 1e-5 * pv[p]
            ls = []
            for sgn in (1.0, -1.0):
                e.reset(gpu_lib.model_with_params(m, *(pv + sgn * h * np.eye(4)[p])))
                ls.append(float(np.sum(e.run_schedule(dts) * w)))
            fd = (ls[0] - ls[1]) / (2 * h)
            assert abs(fd - g[p]) <= 1e-5 * abs(g[p]), (p, fd, g[p])
            live += 1
        assert live >= 3
    finally:
        gpu_lib.set_stop_tolerances()
