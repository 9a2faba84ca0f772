"""Model descriptions for the explicit-dynamics step: meshes, material, boundary conditions, solver.

A :class:`Model` holds what a DynELA ``.dyn`` deck declares before ``END PREPROCESSOR``: nodes,
``ElQua4nAx`` / ``ElHex8n3D`` connectivity, one ``IsoHardElastoplastic`` material, an initial
``BoundarySpeed`` on every node, constant ``BoundaryRestrain`` / ``BoundarySpeed`` groups and the
``ExplicitSolverCH`` settings.  Node and element order is creation order, which the reference
keeps as its internal ``Id`` (finiteElement/Domain.C:1159-1160).

Generators:

* :func:`taylor_axi` -- the axisymmetric Taylor bar of Samples/Taylor/Taylor_Axi_Parametric.dyn:
  nodes row by row, radial index fastest (:45-50), elements (:64-74), initial speed (0, -v, 0)
  (:105-107), base restrained in y (:110-112), axis restrained in x and z (:115-117),
  ExplicitSolverCH with Courant time step (:120-125).
* :func:`taylor_hex` -- the 3D counterpart with ``ElHex8n3D``: a 40x40 Cartesian cross-section grid
  over the bar's bounding square, keeping the cells whose centre lies inside the radius, extruded in
  z; base restrained in z; Pulse time step (hex8 has no Courant length in the reference,
  finiteElement/ElHex8n3D.C:188-192).
* :func:`taylor_batch` -- seeded parameter draws for many independent axisymmetric Taylor bars.
* :func:`taylor_mixed` -- a 3D bar of two element types in one domain: hexahedra at the impact
  end, tetrahedra above.
"""

from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

ELQUA4NAX = 0
ELHEX8N3D = 1
ELQUA4N2D = 2  # plane strain
ELTET4N3D = 3
ELTET10N3D = 4
# not a reference element: ElHex8n3D at its centre with viscous hourglass control
ELHEX8N3D_1PT = 5
NEN_OF = {ELQUA4NAX: 4, ELHEX8N3D: 8, ELQUA4N2D: 4, ELTET4N3D: 4, ELTET10N3D: 10, ELHEX8N3D_1PT: 8}
NIP_OF = {ELQUA4NAX: 4, ELHEX8N3D: 8, ELQUA4N2D: 4, ELTET4N3D: 1, ELTET10N3D: 4, ELHEX8N3D_1PT: 1}

COURANT = 0
PULSE = 1

RESTRAIN = 0
SPEED = 1
# hardening laws: IsoHardElastoplastic (A + B evp^n), no hardening attached (elastic: never
# yields), IsoHardElastoplasticTabular (DiscreteFunction of evp), IsoHardMetafor (P1..P8)
HARD_POWER = 0
HARD_ELASTIC = 1
HARD_TABULAR = 2
HARD_METAFOR = 3


@dataclass
class BCGroup:
    """One constant boundary condition attached to a node set (Structure::attachConstantBC).

    kind RESTRAIN: ``val`` is the 0/1 mask of restrained components (BoundaryRestrain::set).
    kind SPEED: ``val`` is the imposed velocity; components equal to 0 are left free
    (BoundarySpeed::applyConstant, finiteElement/Boundary.C:478-525).
    """

    kind: int
    val: Sequence[float]
    nodes: np.ndarray


@dataclass
class MaterialLaw:
    """One Material with its isotropic hardening (Material.h:61-156 + an IsotropicHardening).

    params: POWER (A, B, n); METAFOR (P1, ..., P8); table_x/table_y: TABULAR, the
    DiscreteFunction's points in ascending evp."""

    young: float
    poisson: float
    density: float
    law: int = HARD_POWER
    params: Sequence[float] = ()
    table_x: Optional[np.ndarray] = None
    table_y: Optional[np.ndarray] = None


@dataclass
class Model:
    etype: int
    coords: np.ndarray  # (N, 3) float64
    conn: np.ndarray  # (E, nen) int64, 0-based node indices
    young: float = 117e9
    poisson: float = 0.35
    density: float = 8930.0
    A: float = 90e6
    B: float = 292e6
    n: float = 0.31
    v0: Sequence[float] = (0.0, 0.0, 0.0)
    bcs: List[BCGroup] = field(default_factory=list)
    tend: float = 80e-6
    rho_b: float = 0.8182
    safety: float = 0.9
    freq: int = 10
    method: int = COURANT
    nsaves: int = 1
    # several materials (Structure::attachMaterialToElements): None = one power-law material from
    # the fields above; elem_material[e] indexes `materials`
    materials: Optional[List[MaterialLaw]] = None
    elem_material: Optional[np.ndarray] = None
    # initial velocity per node (attachInitialBC on node sets), (N, 3); None = v0 everywhere
    initial_velocity: Optional[np.ndarray] = None
    # ELHEX8N3D_1PT only: the viscous hourglass coefficient
    hourglass: float = 0.05
    # further element groups of other types of the same family, [(etype, conn (E_g, nen_g))],
    # numbered after the elements of `conn` in this order (a deck's setDefaultElement +
    # createElement for each further type); etype/conn above are the first group
    groups: Optional[List[Tuple[int, np.ndarray]]] = None

    def material_laws(self) -> List[MaterialLaw]:
        if self.materials:
            return list(self.materials)
        return [MaterialLaw(self.young, self.poisson, self.density, HARD_POWER,
                            (self.A, self.B, self.n))]

    @property
    def extended(self) -> bool:
        return bool(self.materials) or self.elem_material is not None or \
            self.initial_velocity is not None

    @property
    def N(self) -> int:
        return int(self.coords.shape[0])

    def element_groups(self) -> List[Tuple[int, np.ndarray]]:
        """Every element group, the first one included: [(etype, conn)]."""
        return [(self.etype, self.conn)] + list(self.groups or [])

    @property
    def E_all(self) -> int:
        """Elements of all groups."""
        return int(sum(c.shape[0] for _, c in self.element_groups()))

    @property
    def nIP_all(self) -> int:
        """Integration points of all groups."""
        return int(sum(c.shape[0] * NIP_OF[t] for t, c in self.element_groups()))

    @property
    def E(self) -> int:
        return int(self.conn.shape[0])

    @property
    def dim(self) -> int:
        return 2 if self.etype in (ELQUA4NAX, ELQUA4N2D) else 3

    @property
    def nen(self) -> int:
        return {ELHEX8N3D: 8, ELTET10N3D: 10, ELHEX8N3D_1PT: 8}.get(self.etype, 4)

    @property
    def nip(self) -> int:
        return {ELHEX8N3D: 8, ELTET4N3D: 1, ELHEX8N3D_1PT: 1}.get(self.etype, 4)


def taylor_axi(nr: int = 5, nz: int = 50, radius: float = 3.2e-3, length: float = 32.4e-3,
               speed: float = 227.0, A: float = 90e6, B: float = 292e6, n: float = 0.31,
               young: float = 117e9, poisson: float = 0.35, density: float = 8930.0,
               tend: float = 80e-6, freq: int = 10, safety: float = 0.9,
               rho_b: float = 0.8182) -> Model:
    """Axisymmetric Taylor bar, nr radial x nz axial ElQua4nAx elements (x radial, y axial)."""
    dx = radius / nr
    dy = length / nz
    jj, ii = np.meshgrid(np.arange(nz + 1, dtype=np.float64), np.arange(nr + 1, dtype=np.float64),
                         indexing="ij")
    coords = np.zeros(((nr + 1) * (nz + 1), 3))
    coords[:, 0] = (ii * dx).ravel()
    coords[:, 1] = (jj * dy).ravel()
    j, i = np.meshgrid(np.arange(nz), np.arange(nr), indexing="ij")
    n0 = (i + j * (nr + 1)).ravel()
    conn = np.stack([n0, n0 + 1, n0 + nr + 2, n0 + nr + 1], axis=1).astype(np.int64)
    base = np.arange(nr + 1, dtype=np.int64)
    axis = np.arange(0, (nr + 1) * (nz + 1), nr + 1, dtype=np.int64)
    bcs = [BCGroup(RESTRAIN, (0.0, 1.0, 0.0), base), BCGroup(RESTRAIN, (1.0, 0.0, 1.0), axis)]
    return Model(ELQUA4NAX, coords, conn, young, poisson, density, A, B, n,
                 (0.0, -speed, 0.0), bcs, tend, rho_b, safety, freq, COURANT)


def taylor_plane(nr: int = 5, nz: int = 50, **kw) -> Model:
    """Plane-strain Taylor impact: taylor_axi's mesh and boundary conditions on ElQua4n2D
    elements, x = 0 a symmetry plane instead of the axis."""
    return dataclasses.replace(taylor_axi(nr, nz, **kw), etype=ELQUA4N2D)


def taylor_axi_free_surface(nr: int, nz: int) -> np.ndarray:
    """Node ids of taylor_axi(nr, nz)'s free surface: the outer radius (i = nr) and the free end
    (j = nz), node (i, j) = i + j (nr + 1), ascending and without repetition."""
    outer = nr + np.arange(nz + 1, dtype=np.int64) * (nr + 1)
    top = nz * (nr + 1) + np.arange(nr + 1, dtype=np.int64)
    return np.unique(np.concatenate([outer, top]))


def taylor_hex(ncross: int = 40, nz: int = 400, radius: float = 3.2e-3, length: float = 32.4e-3,
               speed: float = 227.0, A: float = 90e6, B: float = 292e6, n: float = 0.31,
               young: float = 117e9, poisson: float = 0.35, density: float = 8930.0,
               tend: float = 80e-6, freq: int = 10, safety: float = 0.9,
               rho_b: float = 0.8182) -> Model:
    """3D Taylor bar of ElHex8n3D: ncross x ncross cells over [-R, R]^2, cells with centre inside R.

    For ncross=40, nz=400 this gives 1264 cells per layer, 505,600 elements and 539,345 nodes.
    Nodes are numbered layer by layer (z slowest), then y, then x; only nodes used by a kept cell
    exist.  Hex node order follows ElHex8n3D (bottom face counter-clockwise, then top face).
    """
    h = 2.0 * radius / ncross
    ci = (np.arange(ncross) + 0.5) * h - radius
    cy, cx = np.meshgrid(ci, ci, indexing="ij")
    keep = (cx * cx + cy * cy) <= radius * radius
    # node grid (ncross+1)^2 per layer; mark the used ones
    used = np.zeros((ncross + 1, ncross + 1), dtype=bool)
    ky, kx = np.nonzero(keep)
    for dy_, dx_ in ((0, 0), (0, 1), (1, 1), (1, 0)):
        used[ky + dy_, kx + dx_] = True
    layer_id = -np.ones((ncross + 1, ncross + 1), dtype=np.int64)
    uy, ux = np.nonzero(used)
    nlayer = uy.size
    layer_id[uy, ux] = np.arange(nlayer)
    gx = ux * h - radius
    gy = uy * h - radius
    dz = length / nz
    coords = np.zeros((nlayer * (nz + 1), 3))
    for k in range(nz + 1):
        coords[k * nlayer:(k + 1) * nlayer, 0] = gx
        coords[k * nlayer:(k + 1) * nlayer, 1] = gy
        coords[k * nlayer:(k + 1) * nlayer, 2] = k * dz
    quad = np.stack([layer_id[ky, kx], layer_id[ky, kx + 1], layer_id[ky + 1, kx + 1],
                     layer_id[ky + 1, kx]], axis=1)
    ncell = quad.shape[0]
    conn = np.zeros((ncell * nz, 8), dtype=np.int64)
    for k in range(nz):
        conn[k * ncell:(k + 1) * ncell, :4] = quad + k * nlayer
        conn[k * ncell:(k + 1) * ncell, 4:] = quad + (k + 1) * nlayer
    base = np.arange(nlayer, dtype=np.int64)
    bcs = [BCGroup(RESTRAIN, (0.0, 0.0, 1.0), base)]
    return Model(ELHEX8N3D, coords, conn, young, poisson, density, A, B, n,
                 (0.0, 0.0, -speed), bcs, tend, rho_b, safety, freq, PULSE)


# the six tetrahedra of a hexahedron around its diagonal 0-6 (node numbering of ElHex8n3D); on a
# grid of hexahedra numbered alike the faces of neighbouring cells are split the same way
_HEX_TO_TETS = ((0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6))
# ElTet10n3D's mid-edge nodes 4..9 (ElTet10n3D.C:37-47)
_TET10_EDGES = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))


def taylor_tet(ncross: int = 8, nz: int = 24, quadratic: bool = False, safety: float = 0.5,
               **kw) -> Model:
    """3D Taylor bar of tetrahedra: each cell of taylor_hex(ncross, nz) split in six (ElTet4n3D),
    or with a node added at the middle of every edge (ElTet10n3D, quadratic=True); base
    restrained in z, Courant time step.  The tetrahedra's Courant length is their shortest edge,
    longer than the stable length of these elements: with the usual safety factor 0.9 the
    reference's own run of this bar inverts elements after ~3 us, hence 0.5."""
    m = taylor_hex(ncross, nz, safety=safety, **kw)
    conn = np.concatenate([m.conn[:, list(t)] for t in _HEX_TO_TETS], axis=0)
    conn = conn.reshape(6, m.E, 4).transpose(1, 0, 2).reshape(-1, 4)  # the tets of a cell together
    coords = m.coords
    etype = ELTET4N3D
    base = m.bcs[0].nodes
    if quadratic:
        ends = np.stack([np.sort(conn[:, list(ed)], axis=1) for ed in _TET10_EDGES], axis=1)
        uniq, inv = np.unique(ends.reshape(-1, 2), axis=0, return_inverse=True)
        mid = m.N + inv.reshape(-1, 6)
        coords = np.concatenate([coords, 0.5 * (coords[uniq[:, 0]] + coords[uniq[:, 1]])])
        conn = np.concatenate([conn, mid], axis=1)
        etype = ELTET10N3D
        base = np.flatnonzero(coords[:, 2] == 0.0).astype(np.int64)
    bcs = [BCGroup(RESTRAIN, (0.0, 0.0, 1.0), base)]
    return dataclasses.replace(m, etype=etype, coords=coords, conn=conn.astype(np.int64), bcs=bcs,
                               method=COURANT)


def taylor_hex_1pt(ncross: int = 40, nz: int = 400, hourglass: float = 0.05, **kw) -> Model:
    """taylor_hex's bar and boundary conditions on the one-point hexahedron with viscous hourglass
    control (ELHEX8N3D_1PT, not a reference element), Courant time step."""
    return dataclasses.replace(taylor_hex(ncross, nz, **kw), etype=ELHEX8N3D_1PT, method=COURANT,
                               hourglass=hourglass)


def taylor_mixed(ncross: int = 6, nz: int = 12, nz_lower: int = 6, lower: int = ELTET4N3D,
                 upper: int = ELTET10N3D, **kw) -> Model:
    """One 3D domain of two element types (Domain::initSolve accepts any mix of one family,
    Domain.C:1042-1060): the cells of taylor_hex(ncross, nz) in the `nz_lower` layers at the
    impact end (z = 0) are of type `lower`, the others of type `upper`; a cell of tetrahedra is
    split in six as in taylor_tet, so the triangles on the interface plane are halves of the faces
    below or above and the two parts share the interface's corner nodes (ElTet10n3D's mid-edge
    nodes there belong to its side only).  Elements of `lower` first, then `upper` (a deck's
    second setDefaultElement); base restrained in z.  Time step: Pulse when a group is ElHex8n3D
    (no Courant length), else Courant with the safety factor of taylor_tet."""
    m = taylor_hex(ncross, nz, **kw)
    ncell = m.E // nz
    layer = np.arange(m.E) // ncell
    coords = m.coords
    groups = []
    for etype, cells in ((lower, m.conn[layer < nz_lower]), (upper, m.conn[layer >= nz_lower])):
        if etype == ELHEX8N3D:
            groups.append((etype, cells.astype(np.int64)))
            continue
        tets = np.stack([cells[:, list(t)] for t in _HEX_TO_TETS], axis=1).reshape(-1, 4)
        if etype == ELTET10N3D:
            ends = np.stack([np.sort(tets[:, list(ed)], axis=1) for ed in _TET10_EDGES], axis=1)
            uniq, inv = np.unique(ends.reshape(-1, 2), axis=0, return_inverse=True)
            mid = coords.shape[0] + inv.reshape(-1, 6)
            coords = np.concatenate([coords, 0.5 * (coords[uniq[:, 0]] + coords[uniq[:, 1]])])
            tets = np.concatenate([tets, mid], axis=1)
        groups.append((etype, tets.astype(np.int64)))
    hexes = ELHEX8N3D in (lower, upper)
    method = PULSE if hexes else COURANT
    safety = kw.get("safety", 0.9 if hexes else 0.5)
    return dataclasses.replace(m, etype=groups[0][0], coords=coords, conn=groups[0][1],
                               groups=groups[1:], method=method, safety=safety)


def tabular_table(A: float, B: float, n: float, step: float = 0.1, stop: float = 10.0):
    """The table a deck builds for IsoHardElastoplasticTabular with a loop
    ``for (eps = 0; eps < stop; eps += step) f.add(eps, A + B * eps^n)`` (Samples/Traction): the
    abscissae accumulate by repeated double additions, as the interpreter does."""
    xs, ys = [], []
    eps = 0.0
    while eps < stop:
        xs.append(eps)
        ys.append(A + B * eps ** n)
        eps += step
    return np.array(xs), np.array(ys)


def impact_two_materials(nr: int = 5, nz: int = 50, radius: float = 3.2e-3,
                         length: float = 32.4e-3, split: float = 0.5, speed: float = 80.0,
                         tend: float = 40e-6, freq: int = 10) -> Model:
    """Axisymmetric bar of two bonded materials in the pattern of Samples/Traction/Traction.dyn:
    the lower part (rows j < split*nz) is the deck's target -- E 74.2 GPa, nu 0.33, rho 2784, an
    IsoHardElastoplasticTabular law tabulating 360 MPa + 316 MPa eps^0.28 every 0.1 up to 10 -- the
    upper part its projectile -- E 193.6 GPa, nu 0.3, rho 7800, no hardening attached (elastic),
    and only the projectile's nodes start at `speed` towards the base; base and axis restrained."""
    m = taylor_axi(nr, nz, radius, length, 0.0, tend=tend, freq=freq)
    tx, ty = tabular_table(360e6, 316e6, 0.28)
    target = MaterialLaw(74.2e9, 0.33, 2784.0, HARD_TABULAR, (), tx, ty)
    projectile = MaterialLaw(193.6e9, 0.3, 7800.0, HARD_ELASTIC, ())
    js = int(round(split * nz))
    row = np.repeat(np.arange(nz), nr)
    em = (row >= js).astype(np.int64)
    v = np.zeros((m.N, 3))
    node_row = np.arange(m.N) // (nr + 1)
    v[node_row >= js, 1] = -speed
    return dataclasses.replace(m, young=74.2e9, poisson=0.33, density=2784.0,
                               materials=[target, projectile], elem_material=em,
                               initial_velocity=v)


def impact_two_materials_hex(ncross: int = 6, nz: int = 12, radius: float = 3.2e-3,
                             length: float = 32.4e-3, split: float = 0.5, speed: float = 80.0,
                             tend: float = 40e-6, freq: int = 10) -> Model:
    """impact_two_materials' bonded pair on taylor_hex's 3D bar of ElHex8n3D, Pulse time step:
    the layers below split*nz are the tabular-hardening target, those above the elastic projectile,
    whose nodes (the interface plane's included) start at `speed` towards the base; the base is
    restrained in z."""
    m = taylor_hex(ncross, nz, radius, length, 0.0, tend=tend, freq=freq)
    tx, ty = tabular_table(360e6, 316e6, 0.28)
    target = MaterialLaw(74.2e9, 0.33, 2784.0, HARD_TABULAR, (), tx, ty)
    projectile = MaterialLaw(193.6e9, 0.3, 7800.0, HARD_ELASTIC, ())
    js = int(round(split * nz))
    dz = length / nz
    em = (m.coords[m.conn[:, 0], 2] >= js * dz - 0.5 * dz).astype(np.int64)  # bottom face's layer
    v = np.zeros((m.N, 3))
    v[m.coords[:, 2] >= js * dz - 0.5 * dz, 2] = -speed
    return dataclasses.replace(m, young=74.2e9, poisson=0.33, density=2784.0,
                               materials=[target, projectile], elem_material=em,
                               initial_velocity=v)


def group_materials(m: Model, laws: Sequence[MaterialLaw]) -> Model:
    """The model with material i on the elements of element group i (element_groups order): a
    domain of several element types whose parts are also of several materials."""
    groups = m.element_groups()
    assert len(laws) == len(groups)
    em = np.concatenate([np.full(c.shape[0], i, dtype=np.int64) for i, (_, c) in enumerate(groups)])
    return dataclasses.replace(m, materials=list(laws), elem_material=em)


def metafor_bar(nr: int = 5, nz: int = 50, speed: float = 227.0, tend: float = 40e-6,
                P=(90e6, 200e6, 10.0, 50e6, 0.5, 1.0, 0.1, 1e8)) -> Model:
    """The copper Taylor bar with an IsoHardMetafor law (P1..P8):
    sigma_y = (P2 - P1)(1 - exp(-P3 evp)) + P4 evp^P5 + P1 (1 + P6 evp)^P7 + P8 evp."""
    m = taylor_axi(nr, nz, speed=speed, tend=tend)
    law = MaterialLaw(m.young, m.poisson, m.density, HARD_METAFOR, tuple(P))
    return dataclasses.replace(m, materials=[law])


def necking_bar(ncross: int = 40, nz: int = 166, radius: float = 6.4e-3, length: float = 53.3e-3,
                speed: float = 1.0, A: float = 90e6, B: float = 292e6, n: float = 0.31,
                young: float = 117e9, poisson: float = 0.35, density: float = 8930.0,
                mass_scaling: float = 100.0, imperfection: float = 0.005,
                tend: float = 10.66e-3, freq: int = 10, safety: float = 0.9,
                rho_b: float = 0.8182) -> Model:
    """3D tensile bar of ElHex8n3D for necking: the cross-section grid of taylor_hex (gauge radius
    6.4 mm, length 53.3 mm; ncross=40, nz=166 gives 1264 cells per layer, 209,824 elements), the
    end z = 0 clamped (BoundaryRestrain 1 1 1), the end z = L pulled at `speed` along z
    (BoundarySpeed 0 0 speed; x and y free), starting at rest.  The radius is reduced by the
    relative `imperfection` around mid-length, r(z) = R (1 - imp exp(-((z - L/2) / (0.1 L))^2)),
    so that the neck forms there.  The density is multiplied by `mass_scaling` (mass scaling: with
    the default 100 the stable step grows tenfold and 30,000 steps of 3.55e-7 s cover the 10.66 ms
    it takes to stretch the bar by 20 % at 1 m/s); copper J2 hardening as the Taylor bars.
    Node numbering as taylor_hex: layer by layer along z."""
    m = taylor_hex(ncross, nz, radius, length, 0.0, A, B, n, young, poisson, density * mass_scaling,
                   tend, freq, safety, rho_b)
    coords = m.coords.copy()
    z = coords[:, 2]
    scale = 1.0 - imperfection * np.exp(-(((z - 0.5 * length) / (0.1 * length)) ** 2))
    coords[:, 0] *= scale
    coords[:, 1] *= scale
    nlayer = m.N // (nz + 1)
    base = np.arange(nlayer, dtype=np.int64)
    top = nz * nlayer + np.arange(nlayer, dtype=np.int64)
    bcs = [BCGroup(RESTRAIN, (1.0, 1.0, 1.0), base), BCGroup(SPEED, (0.0, 0.0, speed), top)]
    return Model(ELHEX8N3D, coords, m.conn, young, poisson, density * mass_scaling, A, B, n,
                 (0.0, 0.0, 0.0), bcs, tend, rho_b, safety, freq, PULSE)


def necking_mid_nodes(model: Model, nz: int) -> np.ndarray:
    """Node ids of the mid-length layer (z = L/2 for even nz) of a necking_bar(.., nz, ..)."""
    nlayer = model.N // (nz + 1)
    k = nz // 2
    return k * nlayer + np.arange(nlayer, dtype=np.int64)


def necking_batch(count: int = 32, seed: int = 0, ncross: int = 40, nz: int = 166,
                  A_range=(60e6, 150e6), B_range=(200e6, 400e6), n_range=(0.2, 0.5)) -> List[Model]:
    """Seeded parameter sets (A, B, n drawn as in taylor_batch) on one necking bar mesh."""
    rng = np.random.default_rng(seed)
    base = necking_bar(ncross, nz)
    out = []
    for _ in range(count):
        A = float(rng.uniform(*A_range))
        B = float(rng.uniform(*B_range))
        nn = float(rng.uniform(*n_range))
        out.append(dataclasses.replace(base, A=A, B=B, n=nn))
    return out


def taylor_batch(count: int = 256, seed: int = 0, nr_range=(4, 40), nz_range=(40, 400),
                 v_range=(150.0, 300.0), A_range=(60e6, 150e6), B_range=(200e6, 400e6),
                 n_range=(0.2, 0.5), tend: float = 80e-6) -> List[Model]:
    """Seeded draws of independent axisymmetric Taylor bars with uneven meshes."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nr = int(rng.integers(nr_range[0], nr_range[1] + 1))
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        v = float(rng.uniform(*v_range))
        A = float(rng.uniform(*A_range))
        B = float(rng.uniform(*B_range))
        nn = float(rng.uniform(*n_range))
        out.append(taylor_axi(nr, nz, speed=v, A=A, B=B, n=nn, tend=tend))
    return out
