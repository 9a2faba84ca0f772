"""The deck-level mirror (dynela.Structure and its companions): a model built by the calls a .dyn
deck makes (Samples/Taylor/Taylor_Axi_Parametric.dyn's statements, the two-material pattern of
Samples/Traction/Traction.dyn, a domain whose default element changes between createElement calls)
is the model the generators in meshes build for the same problem.  No GPU here; the GPU run of a
deck-built model is in test_gpu_deck.py."""

import numpy as np
import pytest

from redynela_gb300 import dynela, meshes


def taylor_axi_deck(nr=5, nz=50, A=90e6, B=292e6, n=0.31, young=117e9, poisson=0.35,
                    density=8930.0, stop=80.0e-6, width=3.2e-3, height=32.4e-3, speed=227.0):
    """Taylor_Axi_Parametric.dyn's statements, with its parameters as arguments."""
    st = dynela.Structure()
    dx, dy = width / nr, height / nz
    cyl = dynela.NodeSet()
    k = 1
    for j in range(nz + 1):
        for i in range(nr + 1):
            st.createNode(k, i * dx, j * dy, 0)
            cyl.add(k)
            k += 1
    nodes = k - 1
    st.setDefaultElement(dynela.ElQua4nAx)
    els = dynela.ElementSet()
    e = 1
    for j in range(nz):
        for i in range(nr):
            x1 = i + j * (nr + 1) + 1
            x2 = i + j * (nr + 1) + 2
            x3 = i + (j + 1) * (nr + 1) + 2
            x4 = i + (j + 1) * (nr + 1) + 1
            st.createElement(e, x1, x2, x3, x4)
            els.add(e)
            e += 1
    mat = dynela.Material()
    hard = dynela.IsoHardElastoplastic()
    hard.setYieldStress(A)
    hard.setHardParameter(B)
    hard.setHardExponent(n)
    st.addMaterial(mat)
    mat.setYoung(young)
    mat.setPoisson(poisson)
    mat.setDensity(density)
    mat.setColor(1, 0, 1)
    mat.setHardening(hard)
    base = dynela.NodeSet()
    base.add(1, nr + 1)
    axis = dynela.NodeSet()
    axis.add(1, nodes, nr + 1)
    st.attachMaterialToElements(mat, els)
    ini = dynela.BoundarySpeed()
    ini.set(0, -speed, 0)
    st.attachInitialBC(ini, cyl)
    bd = dynela.BoundaryRestrain()
    bd.set(0, 1, 0)
    st.attachConstantBC(bd, base)
    ad = dynela.BoundaryRestrain()
    ad.set(1, 0, 1)
    st.attachConstantBC(ad, axis)
    solver = dynela.ExplicitSolverCH()
    solver.setTimes(0, stop)
    st.setSaveTimes(0, stop, stop / 20)
    st.addSolver(solver)
    solver.setTimeStepMethod("Courant")
    return st, {"els": els, "nodes": cyl, "nr": nr, "nz": nz}


def assert_same_model(a, b):
    assert a.etype == b.etype and a.method == b.method
    assert np.array_equal(a.coords, b.coords) and np.array_equal(a.conn, b.conn)
    assert [(g.kind, tuple(g.val), list(g.nodes)) for g in a.bcs] == \
           [(g.kind, tuple(g.val), list(g.nodes)) for g in b.bcs]
    for f in ("tend", "rho_b", "safety", "freq"):
        assert getattr(a, f) == getattr(b, f), f
    la, lb = a.material_laws(), b.material_laws()
    assert len(la) == len(lb)
    for x, y in zip(la, lb):
        assert (x.young, x.poisson, x.density, x.law, tuple(x.params)) == \
               (y.young, y.poisson, y.density, y.law, tuple(y.params))
        if x.law == meshes.HARD_TABULAR:
            assert np.array_equal(x.table_x, y.table_x) and np.array_equal(x.table_y, y.table_y)
    ea = a.elem_material if a.elem_material is not None else np.zeros(a.E_all, dtype=np.int64)
    eb = b.elem_material if b.elem_material is not None else np.zeros(b.E_all, dtype=np.int64)
    assert np.array_equal(ea, eb)
    va = a.initial_velocity if a.initial_velocity is not None else np.tile(a.v0, (a.N, 1))
    vb = b.initial_velocity if b.initial_velocity is not None else np.tile(b.v0, (b.N, 1))
    assert np.array_equal(va, vb)
    ga, gb = a.element_groups(), b.element_groups()
    assert [t for t, _ in ga] == [t for t, _ in gb]
    assert all(np.array_equal(x, y) for (_, x), (_, y) in zip(ga, gb))


def test_taylor_deck_is_the_generators_bar():
    st, _ = taylor_axi_deck(5, 50)
    assert_same_model(st.model(), meshes.taylor_axi(5, 50))


def test_two_material_deck_is_the_generators_impact():
    """The Traction pattern: a tabular-hardening target on the lower rows (an
    IsoHardElastoplasticTabular over a DiscreteFunction), an elastic projectile (no hardening) on
    the upper rows, the initial speed on the projectile's nodes only."""
    nr, nz, js = 5, 50, 25
    st, sets = taylor_axi_deck(nr, nz, speed=0.0, stop=40e-6)
    ref = meshes.impact_two_materials(nr, nz)
    st._materials.clear()
    st._initial.clear()
    target, proj = dynela.Material(), dynela.Material()
    target.setYoung(74.2e9)
    target.setPoisson(0.33)
    target.setDensity(2784.0)
    fn = dynela.DiscreteFunction()
    tx, ty = meshes.tabular_table(360e6, 316e6, 0.28)
    for x, y in zip(tx[::-1], ty[::-1]):  # any insertion order: the function keeps x sorted
        fn.add(x, y)
    tab = dynela.IsoHardElastoplasticTabular()
    tab.setFunction(fn)
    target.setHardening(tab)
    proj.setYoung(193.6e9)
    proj.setPoisson(0.3)
    proj.setDensity(7800.0)
    low, up = dynela.ElementSet(), dynela.ElementSet()
    low.add(1, js * nr)
    up.add(js * nr + 1, nz * nr)
    st.attachMaterialToElements(target, low)
    st.attachMaterialToElements(proj, up)
    moving = dynela.NodeSet()
    moving.add(js * (nr + 1) + 1, (nz + 1) * (nr + 1))
    v = dynela.BoundarySpeed()
    v.set(0, -80.0, 0)
    st.attachInitialBC(v, moving)
    assert_same_model(st.model(), ref)


def test_deck_switching_the_default_element_makes_groups():
    """Tetrahedra created first, then hexahedra after setDefaultElement(ElHex8n3D): two element
    groups in creation order, as meshes.taylor_mixed builds them; the last material attached to
    an element wins; a node set's imposed speed becomes a BoundarySpeed group."""
    ref = meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D, upper=meshes.ELHEX8N3D)
    st = dynela.Structure()
    for i, x in enumerate(ref.coords):
        st.createNode(i + 1, *x)
    num = 1
    all_els = dynela.ElementSet()
    for etype, conn in ref.element_groups():
        st.setDefaultElement(etype)
        for row in conn:
            st.createElement(num, *(row + 1))
            all_els.add(num)
            num += 1
    m0, m1 = dynela.Material(), dynela.Material()
    for m, A in ((m0, 1e6), (m1, ref.A)):
        h = dynela.IsoHardElastoplastic()
        h.setYieldStress(A)
        h.setHardParameter(ref.B)
        h.setHardExponent(ref.n)
        m.setYoung(ref.young)
        m.setPoisson(ref.poisson)
        m.setDensity(ref.density)
        m.setHardening(h)
    st.attachMaterialToElements(m0, all_els)
    st.attachMaterialToElements(m1, all_els)  # replaces m0 everywhere
    allnodes = dynela.NodeSet()
    allnodes.add(1, ref.N)
    ini = dynela.BoundarySpeed()
    ini.set(*ref.v0)
    st.attachInitialBC(ini, allnodes)
    for g in ref.bcs:
        ns = dynela.NodeSet()
        for k in g.nodes:
            ns.add(int(k) + 1)
        b = dynela.BoundaryRestrain() if g.kind == meshes.RESTRAIN else dynela.BoundarySpeed()
        b.set(*g.val)
        st.attachConstantBC(b, ns)
    pull = dynela.BoundarySpeed()
    pull.set(0, 0, 1.0)
    top = dynela.NodeSet()
    top.add(ref.N)
    st.attachConstantBC(pull, top)
    s = dynela.ExplicitSolverCH()
    s.setTimes(0, ref.tend)
    s.setTimeStepMethod("Pulse")
    st.addSolver(s)
    m = st.model()
    assert m.materials is None and m.A == ref.A  # one power-law material after the replacement
    assert m.bcs[-1].kind == meshes.SPEED and list(m.bcs[-1].nodes) == [ref.N - 1]
    m.bcs = m.bcs[:-1]
    assert_same_model(m, ref)


def test_deck_errors():
    st = dynela.Structure()
    with pytest.raises(ValueError):
        st.createElement(1, 1, 2, 3, 4)  # no default element
    s = dynela.ExplicitSolverCH()
    with pytest.raises(ValueError):
        s.setTimeStepMethod("Unknown")
    with pytest.raises(ValueError):
        s.setDissipation(1.5)
