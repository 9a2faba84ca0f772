"""dnl_internal_forces_static, the internal-force entry point for callers that cannot allocate
device memory: a framework whose memory manager owns every device byte and forbids libraries their
own cudaMalloc, or a process with a device budget fixed before the solver starts.  The test plays
such a caller: it allocates every input and output itself (through torch), hands the device
pointers to the library, and checks the result against the handle-based dnl_internal_forces on the
same state, on two calls in a row (the second sees the library's fixed scratch array as the first
left it), for every element type the entry point accepts.  It also checks the error path: an
inverted element gives DNL_ERR_NEG_DETJ with that element's index, and the next valid call on the
same arrays returns 0 with no element reported.  Tolerance: the one the parity tests use, 1e-12
relative.  This file sorts last so that a run stopping at its first failure has run every other
test before it."""

import ctypes as C

import numpy as np
import pytest

from oracle import states
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_ELEMENT_DOFS = 1 << 20
DNL_ERR_NEG_DETJ = 1
DNL_ERR_ARG = 6


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


def _ns(m):
    return 6 if m.dim == 3 else 4


def _ip_array(m, st):
    """The documented layout: S | Eps | EpsPlas (ns symmetric components each) | p | evp | evp^n."""
    ns = _ns(m)
    nI = m.E * m.nip
    comps = []
    for name in ("S", "Eps", "EpsPlas"):
        t = np.asarray(st[name]).reshape(nI, 3, 3)
        comps += [t[:, i, j] for i, j in SYM[:ns]]
    evp = np.asarray(st["evp"]).ravel()
    comps += [np.asarray(st["p"]).ravel(), evp, evp ** m.n]
    return np.stack(comps)


def _csr(conn, N):
    E, nen = conn.shape
    start = np.zeros(N + 1, dtype=np.int32)
    np.add.at(start, conn.ravel() + 1, 1)
    start = np.cumsum(start).astype(np.int32)
    entry = np.zeros(E * nen, dtype=np.int32)
    fill = start[:-1].copy()
    for e in range(E):
        for k in range(nen):
            n = conn[e, k]
            entry[fill[n]] = e * nen + k
            fill[n] += 1
    return start, entry


def _model(etype):
    if etype == meshes.ELQUA4NAX:
        return meshes.taylor_axi(8, 30)
    if etype == meshes.ELQUA4N2D:
        return meshes.taylor_plane(8, 30)
    if etype == meshes.ELHEX8N3D:
        return meshes.taylor_hex(6, 10)
    if etype == meshes.ELTET4N3D:
        return meshes.taylor_tet(4, 8)
    return meshes.taylor_tet(3, 4, quadratic=True)


class Caller:
    """A caller that owns all device memory: torch tensors, their addresses passed to the library."""

    def __init__(self, gpu_lib, m, conn):
        import torch
        self.torch = torch
        self.m = m
        self.dev = torch.device("cuda")
        start, entry = _csr(conn, m.N)
        self.conn = torch.tensor(np.ascontiguousarray(conn.T), dtype=torch.int32, device=self.dev)
        self.start = torch.tensor(start, device=self.dev)
        self.entry = torch.tensor(entry, device=self.dev)
        self.fint = torch.zeros(m.N * m.dim, dtype=torch.float64, device=self.dev)
        self.L = gpu_lib.lib()
        self.L.dnl_internal_forces_static.argtypes = [C.POINTER(StaticArgs), C.c_void_p,
                                                      C.POINTER(C.c_int)]
        self.L.dnl_internal_forces_static.restype = C.c_int

    def call(self, ip, x, u):
        t = self.torch
        m = self.m
        t_x = t.tensor(np.ascontiguousarray(np.asarray(x).T), dtype=t.float64, device=self.dev)
        t_u = t.tensor(np.ascontiguousarray(np.asarray(u).T), dtype=t.float64, device=self.dev)
        t.cuda.synchronize()
        args = StaticArgs(m.etype, m.N, m.E, self.conn.data_ptr(), self.start.data_ptr(),
                          self.entry.data_ptr(), t_x.data_ptr(), t_u.data_ptr(), ip.data_ptr(),
                          self.fint.data_ptr(), m.young, m.poisson, m.density, m.A, m.B, m.n)
        bad = C.c_int(12345)
        rc = self.L.dnl_internal_forces_static(C.byref(args), None, C.byref(bad))
        return rc, bad.value


@pytest.mark.parametrize("etype", [meshes.ELQUA4NAX, meshes.ELQUA4N2D, meshes.ELHEX8N3D,
                                   meshes.ELTET4N3D, meshes.ELTET10N3D],
                         ids=["axi", "plane", "hex8", "tet4", "tet10"])
def test_static_entry_matches_handle_path_twice(gpu_lib, etype):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("torch sees no CUDA device")
    m = _model(etype)
    assert m.E * m.nen * m.dim <= MAX_ELEMENT_DOFS
    st = states.random_state(m, seed=31)
    rng = np.random.default_rng(5)
    x = m.coords[m.conn]
    h = float(np.min(np.linalg.norm(x[:, 1] - x[:, 0], axis=1)))
    du2 = np.zeros((m.N, 3))
    du2[:, :m.dim] = rng.normal(scale=1e-3 * h, size=(m.N, m.dim))
    coords2 = st["coords"] + du2

    # the existing entry point (a handle, allocated by the library)
    d = gpu_lib.GpuDomain(m)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    ref = []
    for xx, u in ((st["coords"], st["du"]), (coords2, du2)):
        f = d.internal_forces(coords=xx, du=u, dt=st["dt"])
        ref.append((f, d.get_state("S", "Eps", "EpsPlas", "p", "evp")))
    d.close()

    # the static entry point: every buffer allocated by the caller
    caller = Caller(gpu_lib, m, m.conn)
    t_ip = torch.tensor(_ip_array(m, st), dtype=torch.float64, device=caller.dev)
    ns = _ns(m)
    for call, (xx, u) in enumerate(((st["coords"], st["du"]), (coords2, du2))):
        rc, bad = caller.call(t_ip, xx, u)
        assert rc == 0 and bad == -1, (call, rc, bad)
        f_ref, s_ref = ref[call]
        assert rel(caller.fint.cpu().numpy(), f_ref) <= TOL, call
        ip = t_ip.cpu().numpy()
        for base, name in ((0, "S"), (ns, "Eps"), (2 * ns, "EpsPlas")):
            for k, (i, j) in enumerate(SYM[:ns]):
                assert rel(ip[base + k], s_ref[name][:, :, i, j].ravel()) <= TOL, (call, name, k)
        assert rel(ip[3 * ns], s_ref["p"].ravel()) <= TOL
        assert rel(ip[3 * ns + 1], s_ref["evp"].ravel()) <= TOL


def test_static_entry_reports_inverted_element_then_recovers(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("torch sees no CUDA device")
    m = meshes.taylor_axi(4, 12)
    st = states.random_state(m, seed=3)
    bad_e = 17
    inverted = m.conn.copy()
    inverted[bad_e] = inverted[bad_e][[0, 3, 2, 1]]  # clockwise: negative Jacobian

    caller = Caller(gpu_lib, m, inverted)
    t_ip = torch.tensor(_ip_array(m, st), dtype=torch.float64, device=caller.dev)
    rc, bad = caller.call(t_ip, st["coords"], st["du"])
    assert rc == DNL_ERR_NEG_DETJ and bad == bad_e, (rc, bad)

    # the same arrays (scratch and error word as the failed call left them), a valid mesh
    good = Caller(gpu_lib, m, m.conn)
    t_ip = torch.tensor(_ip_array(m, st), dtype=torch.float64, device=good.dev)
    rc, bad = good.call(t_ip, st["coords"], st["du"])
    assert rc == 0 and bad == -1, (rc, bad)
    d = gpu_lib.GpuDomain(m)
    d.set_state(S=st["S"], Eps=st["Eps"], EpsPlas=st["EpsPlas"], p=st["p"], evp=st["evp"])
    f_ref = d.internal_forces(coords=st["coords"], du=st["du"], dt=st["dt"])
    d.close()
    assert rel(good.fint.cpu().numpy(), f_ref) <= TOL


def test_static_entry_rejects_oversize_mesh(gpu_lib):
    L = gpu_lib.lib()
    L.dnl_internal_forces_static.argtypes = [C.POINTER(StaticArgs), C.c_void_p, C.POINTER(C.c_int)]
    too_many = MAX_ELEMENT_DOFS // (8 * 3) + 1
    args = StaticArgs(meshes.ELHEX8N3D, 10, too_many, 1, 1, 1, 1, 1, 1, 1,
                      117e9, 0.35, 8930.0, 90e6, 292e6, 0.31)
    bad = C.c_int(0)
    assert L.dnl_internal_forces_static(C.byref(args), None, C.byref(bad)) == DNL_ERR_ARG
    assert bad.value == -1
