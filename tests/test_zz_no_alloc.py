"""dnl_internal_forces_static, the internal-force entry point for callers that cannot allocate
device memory (inside a CUDA stream capture, or under a memory manager that owns all device
memory).  The test plays such a caller: it allocates every input and output itself (through
torch), hands the device pointers to the library, and checks the result against the handle-based
dnl_internal_forces on the same state, on two calls in a row (the second sees the scratch array
as the first left it).  Tolerance: the one the parity tests use, 1e-12 relative."""

import ctypes as C

import numpy as np
import pytest

from oracle import states
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_ELEMENT_DOFS = 1 << 20


class StaticArgs(C.Structure):
    _fields_ = [("etype", C.c_int), ("num_nodes", C.c_int), ("num_elements", C.c_int),
                ("conn", C.c_void_p), ("node_start", C.c_void_p), ("node_entry", C.c_void_p),
                ("coords", C.c_void_p), ("du", C.c_void_p), ("ip", C.c_void_p),
                ("fint", C.c_void_p),
                ("young", C.c_double), ("poisson", C.c_double), ("density", C.c_double),
                ("A", C.c_double), ("B", C.c_double), ("n", C.c_double)]


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


SYM = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def _ip_array(m, st):
    ns = 6 if m.etype == meshes.ELHEX8N3D else 4
    nI = m.E * m.nip
    comps = []
    for name in ("S", "Eps", "EpsPlas"):
        t = np.asarray(st[name]).reshape(nI, 3, 3)
        comps += [t[:, i, j] for i, j in SYM[:ns]]
    evp = np.asarray(st["evp"]).ravel()
    comps += [np.asarray(st["p"]).ravel(), evp, evp ** m.n]
    return np.stack(comps)


def _csr(m):
    start = np.zeros(m.N + 1, dtype=np.int32)
    np.add.at(start, m.conn.ravel() + 1, 1)
    start = np.cumsum(start).astype(np.int32)
    entry = np.zeros(m.E * m.nen, dtype=np.int32)
    fill = start[:-1].copy()
    for e in range(m.E):
        for k in range(m.nen):
            n = m.conn[e, k]
            entry[fill[n]] = e * m.nen + k
            fill[n] += 1
    return start, entry


@pytest.mark.parametrize("etype", [meshes.ELQUA4NAX, meshes.ELHEX8N3D])
def test_static_entry_matches_handle_path_twice(gpu_lib, etype):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("torch sees no CUDA device")
    m = meshes.taylor_axi(8, 30) if etype == meshes.ELQUA4NAX else meshes.taylor_hex(6, 10)
    assert m.E * m.nen * m.dim <= MAX_ELEMENT_DOFS
    st = states.random_state(m, seed=31)
    rng = np.random.default_rng(5)
    h = float(np.min(np.linalg.norm(m.coords[m.conn[:, 1]] - m.coords[m.conn[:, 0]], axis=1)))
    du2 = np.zeros((m.N, 3))
    du2[:, :m.dim] = rng.normal(scale=1e-3 * h, size=(m.N, m.dim))
    coords2 = st["coords"] + du2

    # the existing entry point (a handle, allocated by the library)
    d = gpu_lib.GpuDomain(m)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    ref = []
    for x, u in ((st["coords"], st["du"]), (coords2, du2)):
        f = d.internal_forces(coords=x, du=u, dt=st["dt"])
        ref.append((f, d.get_state("S", "Eps", "EpsPlas", "p", "evp")))

    # the static entry point: every buffer allocated by the caller
    dev = torch.device("cuda")
    start, entry = _csr(m)
    t_conn = torch.tensor(np.ascontiguousarray(m.conn.T), dtype=torch.int32, device=dev)
    t_start = torch.tensor(start, device=dev)
    t_entry = torch.tensor(entry, device=dev)
    t_ip = torch.tensor(_ip_array(m, st), dtype=torch.float64, device=dev)
    t_fint = torch.zeros(m.N * m.dim, dtype=torch.float64, device=dev)
    L = gpu_lib.lib()
    L.dnl_internal_forces_static.argtypes = [C.POINTER(StaticArgs), C.c_void_p, C.POINTER(C.c_int)]
    ns = 6 if etype == meshes.ELHEX8N3D else 4
    for call, (x, u) in enumerate(((st["coords"], st["du"]), (coords2, du2))):
        t_x = torch.tensor(np.ascontiguousarray(np.asarray(x).T), dtype=torch.float64, device=dev)
        t_u = torch.tensor(np.ascontiguousarray(np.asarray(u).T), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        args = StaticArgs(etype, m.N, m.E, t_conn.data_ptr(), t_start.data_ptr(),
                          t_entry.data_ptr(), t_x.data_ptr(), t_u.data_ptr(), t_ip.data_ptr(),
                          t_fint.data_ptr(), m.young, m.poisson, m.density, m.A, m.B, m.n)
        bad = C.c_int(0)
        rc = L.dnl_internal_forces_static(C.byref(args), None, C.byref(bad))
        assert rc == 0, (call, rc, bad.value)
        f_ref, s_ref = ref[call]
        assert rel(t_fint.cpu().numpy(), f_ref) <= TOL, call
        ip = t_ip.cpu().numpy()
        for base, name in ((0, "S"), (ns, "Eps"), (2 * ns, "EpsPlas")):
            for k, (i, j) in enumerate(SYM[:ns]):
                assert rel(ip[base + k], s_ref[name][:, :, i, j].ravel()) <= TOL, (call, name, k)
        assert rel(ip[3 * ns], s_ref["p"].ravel()) <= TOL
        assert rel(ip[3 * ns + 1], s_ref["evp"].ravel()) <= TOL


def test_static_entry_rejects_oversize_mesh(gpu_lib):
    L = gpu_lib.lib()
    L.dnl_internal_forces_static.argtypes = [C.POINTER(StaticArgs), C.c_void_p, C.POINTER(C.c_int)]
    too_many = MAX_ELEMENT_DOFS // (8 * 3) + 1
    args = StaticArgs(meshes.ELHEX8N3D, 10, too_many, 1, 1, 1, 1, 1, 1, 1,
                      117e9, 0.35, 8930.0, 90e6, 292e6, 0.31)
    bad = C.c_int(0)
    assert L.dnl_internal_forces_static(C.byref(args), None, C.byref(bad)) == 6  # DNL_ERR_ARG
