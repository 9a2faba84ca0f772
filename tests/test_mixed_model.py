"""Host side of domains with several element types (no GPU): the mixed bar generator, the model file
the reference harness reads for such a domain (element type 9: each element's own type, then each
element's nodes), and the per-integration-point state arrays that cover every group in element
order.  The GPU side is in test_gpu_mixed.py."""

import struct
import tempfile

import numpy as np

from oracle import dnl_io, states
from redynela_gb300 import meshes


def test_mixed_bar_groups_share_the_interface_nodes():
    m = meshes.taylor_mixed(4, 6, nz_lower=3, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D)
    (t0, c0), (t1, c1) = m.element_groups()
    assert (t0, t1) == (meshes.ELHEX8N3D, meshes.ELTET4N3D)
    assert c0.shape[1] == 8 and c1.shape[1] == 4 and c1.shape[0] == 6 * c0.shape[0]
    # every node belongs to an element, and the interface plane's nodes to both parts
    used = np.zeros(m.N, dtype=bool)
    used[c0.ravel()] = used[c1.ravel()] = True
    assert used.all()
    z = m.coords[:, 2]
    zi = np.max(z[c0.ravel()])
    shared = np.intersect1d(c0.ravel(), c1.ravel())
    assert shared.size > 0 and np.all(z[shared] == zi)
    # tetrahedra are right-handed (positive volume), as the hexahedra's split
    x = m.coords[c1]
    vol = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
    assert np.all(vol > 0)
    assert m.E_all == c0.shape[0] + c1.shape[0] and m.nIP_all == 8 * c0.shape[0] + c1.shape[0]
    assert m.method == meshes.PULSE  # ElHex8n3D has no Courant length


def test_tet10_upper_part_adds_mid_edge_nodes():
    m = meshes.taylor_mixed(4, 6, nz_lower=3)  # ElTet4n3D below, ElTet10n3D above
    (t0, c0), (t1, c1) = m.element_groups()
    assert (t0, t1) == (meshes.ELTET4N3D, meshes.ELTET10N3D) and c1.shape[1] == 10
    mid = 0.5 * (m.coords[c1[:, 0]] + m.coords[c1[:, 1]])
    assert np.array_equal(m.coords[c1[:, 4]], mid)
    assert m.method == meshes.COURANT and m.safety == 0.5


def test_model_file_of_a_mixed_domain():
    m = meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D, upper=meshes.ELHEX8N3D)
    with tempfile.NamedTemporaryFile(suffix=".dnlm") as f:
        dnl_io.write_model(f.name, m)
        data = open(f.name, "rb").read()
    magic, etype, N, E = struct.unpack_from("<4q", data, 0)
    assert magic == dnl_io.MODEL_MAGIC and etype == dnl_io.MIXED and N == m.N and E == m.E_all
    pos = 32 + 8 * 3 * N
    types = np.frombuffer(data, dtype="<i8", count=E, offset=pos)
    assert np.array_equal(types, np.concatenate([np.full(c.shape[0], t) for t, c in m.element_groups()]))
    pos += 8 * E
    nconn = sum(c.size for _, c in m.element_groups())
    conn = np.frombuffer(data, dtype="<i8", count=nconn, offset=pos)
    assert np.array_equal(conn, np.concatenate([c.ravel() for _, c in m.element_groups()]))
    # the material record follows the connectivity
    young = struct.unpack_from("<d", data, pos + 8 * nconn)[0]
    assert young == m.young


def test_random_state_covers_every_group():
    m = meshes.taylor_mixed(4, 3, nz_lower=1, lower=meshes.ELTET4N3D, upper=meshes.ELHEX8N3D)
    st = states.random_state(m, seed=3)
    n = m.nIP_all
    assert st["S"].shape == (n, 3, 3) and st["p"].shape == (n,) and st["evp"].shape == (n,)
    assert np.allclose(st["S"], np.swapaxes(st["S"], -1, -2))
    assert np.allclose(np.trace(st["S"], axis1=-2, axis2=-1), 0.0, atol=1e-3)


def test_group_materials_assign_one_material_per_group():
    a = meshes.MaterialLaw(117e9, 0.35, 8930.0)
    b = meshes.MaterialLaw(193.6e9, 0.3, 7800.0)
    m = meshes.group_materials(meshes.taylor_mixed(4, 6, nz_lower=3), [a, b])
    (_, c0), (_, c1) = m.element_groups()
    assert m.elem_material.shape == (m.E_all,)
    assert np.all(m.elem_material[:c0.shape[0]] == 0) and np.all(m.elem_material[c0.shape[0]:] == 1)
    assert m.material_laws() == [a, b]


def test_two_material_hex_bar_layers_and_speeds():
    """impact_two_materials_hex: the lower half of the layers is the target (material 0), the upper
    half the projectile, whose nodes (the interface plane's included) alone move."""
    m = meshes.impact_two_materials_hex(4, 12)
    z_bottom = m.coords[m.conn[:, 0], 2]
    zi = 6 * (m.coords[:, 2].max() / 12)
    assert np.all(m.elem_material[z_bottom < zi - 1e-12] == 0)
    assert np.all(m.elem_material[z_bottom >= zi - 1e-12] == 1)
    moving = m.initial_velocity[:, 2] != 0
    assert np.all(m.coords[moving, 2] >= zi - 1e-12) and np.all(m.coords[~moving, 2] < zi - 1e-12)
    assert m.method == meshes.PULSE and len(m.material_laws()) == 2
