"""ctypes binding of the C oracle (oracle/liboracle.so) -- test infrastructure only.

The oracle restates DynELA's explicit step on the CPU (oracle/dnl_oracle.c).  Tests compare the
GPU library against it; bench.py times it as the CPU baseline.  The product never imports this.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SENS_PATH = os.path.join(HERE, "libsens.so")

_lib = None
_sens = None


def _stale(out, src):
    return not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(os.path.join(HERE, src))


def build(force: bool = False) -> str:
    if (force or _stale(LIB_PATH, "dnl_oracle.c") or _stale(SENS_PATH, "dnl_sens.cc")
            or _stale(LIB_PATH, "tet10_tables.h") or _stale(SENS_PATH, "tet10_tables.h")):
        subprocess.run(["make", "-C", HERE, "port"], check=True, capture_output=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp, lp = C.POINTER(C.c_double), C.POINTER(C.c_long)
        L.dnlo_create.restype = C.c_void_p
        L.dnlo_create.argtypes = [C.c_int, C.c_long, C.c_long, dp, lp, dp, dp, C.c_long, lp, dp,
                                  lp, lp, dp]
        L.dnlo_destroy.argtypes = [C.c_void_p]
        L.dnlo_array.restype = dp
        L.dnlo_array.argtypes = [C.c_void_p, C.c_char_p, lp]
        L.dnlo_get.restype = C.c_double
        L.dnlo_get.argtypes = [C.c_void_p, C.c_char_p]
        L.dnlo_set.argtypes = [C.c_void_p, C.c_char_p, C.c_double]
        for fn in ("dnlo_internal_forces", "dnlo_mass", "dnlo_prologue", "dnlo_bad_element"):
            getattr(L, fn).argtypes = [C.c_void_p]
        L.dnlo_internal_matrices.argtypes = [C.c_void_p, C.c_int]
        L.dnlo_time_step.argtypes = [C.c_void_p, C.c_int]
        L.dnlo_courant.restype = C.c_double
        L.dnlo_courant.argtypes = [C.c_void_p]
        L.dnlo_max_frequency.argtypes = [C.c_void_p, dp]
        L.dnlo_steps.argtypes = [C.c_void_p, C.c_long, lp]
        L.dnlo_set_threads.argtypes = [C.c_int]
        L.dnlo_tables.argtypes = [C.c_int, dp, dp]
        L.dnlo_set_materials.argtypes = [C.c_void_p, C.c_int, dp, lp, dp, dp, lp]
        L.dnlo_set_velocity.argtypes = [C.c_void_p, dp]
        L.dnlo_set_hourglass.argtypes = [C.c_void_p, C.c_double]
        _lib = L
    return _lib


def tables(etype: int):
    """(N, dN/dxi) tables the oracle builds: (nip, nen) and (nip, nen, dim)."""
    nen = {1: 8, 4: 10}.get(etype, 4)
    nip = {1: 8, 3: 1}.get(etype, 4)
    dim = 2 if etype in (0, 2) else 3
    N = np.zeros((nip, nen))
    dN = np.zeros((nip, nen, dim))
    lib().dnlo_tables(etype, _dp(N), _dp(dN))
    return N, dN


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _lp(a):
    return a.ctypes.data_as(C.POINTER(C.c_long))


class OracleError(RuntimeError):
    def __init__(self, code, elem):
        super().__init__(f"oracle status {code} (element {elem})")
        self.code = code
        self.elem = elem


class Oracle:
    """One model on the CPU oracle.  Arrays are live views into the C state."""

    def __init__(self, model, threads: int = 0):
        L = lib()
        if threads:
            L.dnlo_set_threads(int(threads))
        m = model
        coords = np.ascontiguousarray(m.coords, dtype=np.float64)
        conn = np.ascontiguousarray(m.conn, dtype=np.int64)
        mat = np.array([m.young, m.poisson, m.density, m.A, m.B, m.n], dtype=np.float64)
        v0 = np.array(m.v0, dtype=np.float64)
        kinds = np.array([g.kind for g in m.bcs] or [0], dtype=np.int64)
        vals = np.array([list(g.val) for g in m.bcs] or [[0, 0, 0]], dtype=np.float64).ravel()
        starts = np.zeros(len(m.bcs) + 1, dtype=np.int64)
        for i, g in enumerate(m.bcs):
            starts[i + 1] = starts[i] + len(g.nodes)
        nodes = np.concatenate([np.asarray(g.nodes, dtype=np.int64) for g in m.bcs]) if m.bcs \
            else np.zeros(1, dtype=np.int64)
        solver = np.array([m.tend, m.rho_b, m.safety, float(m.freq), float(m.method)],
                          dtype=np.float64)
        self._keep = (coords, conn, mat, v0, kinds, vals, starts, nodes, solver)
        self.h = L.dnlo_create(m.etype, m.N, m.E, _dp(coords), _lp(conn), _dp(mat), _dp(v0),
                               len(m.bcs), _lp(kinds), _dp(vals), _lp(starts), _lp(nodes),
                               _dp(solver))
        if not self.h:
            raise ValueError("dnlo_create rejected the model")
        self.model = m
        self.L = L
        if getattr(m, "extended", False):
            self._apply_extensions(m)
        if m.etype == 5:
            L.dnlo_set_hourglass(self.h, float(m.hourglass))

    def _apply_extensions(self, m):
        laws = m.material_laws()
        props = np.zeros((len(laws), 12))
        starts = np.zeros(len(laws) + 1, dtype=np.int64)
        xs, ys = [], []
        for i, ml in enumerate(laws):
            props[i, :4] = (ml.young, ml.poisson, ml.density, ml.law)
            props[i, 4:4 + len(ml.params)] = ml.params
            tx = np.zeros(0) if ml.table_x is None else np.asarray(ml.table_x, dtype=np.float64)
            ty = np.zeros(0) if ml.table_y is None else np.asarray(ml.table_y, dtype=np.float64)
            xs.append(tx)
            ys.append(ty)
            starts[i + 1] = starts[i] + tx.size
        tx = np.concatenate(xs) if starts[-1] else np.zeros(1)
        ty = np.concatenate(ys) if starts[-1] else np.zeros(1)
        em = None if m.elem_material is None else np.ascontiguousarray(m.elem_material, dtype=np.int64)
        self._keep_ext = (props, starts, tx, ty, em)
        r = self.L.dnlo_set_materials(self.h, len(laws), _dp(props), _lp(starts), _dp(tx), _dp(ty),
                                      _lp(em) if em is not None else None)
        if r:
            raise ValueError(f"dnlo_set_materials: {r}")
        if m.initial_velocity is not None:
            v = np.ascontiguousarray(m.initial_velocity, dtype=np.float64)
            self._keep_v = v
            self.L.dnlo_set_velocity(self.h, _dp(v))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.dnlo_destroy(self.h)
            self.h = None

    def array(self, name: str) -> np.ndarray:
        cnt = C.c_long(0)
        p = self.L.dnlo_array(self.h, name.encode(), C.byref(cnt))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(cnt.value,))

    def get(self, name: str) -> float:
        return self.L.dnlo_get(self.h, name.encode())

    def set(self, name: str, value: float) -> None:
        if self.L.dnlo_set(self.h, name.encode(), float(value)):
            raise KeyError(name)

    def _check(self, rc):
        if rc:
            raise OracleError(rc, self.L.dnlo_bad_element(self.h))

    def internal_matrices(self, reference: bool = False):
        self._check(self.L.dnlo_internal_matrices(self.h, int(reference)))

    def internal_forces(self) -> np.ndarray:
        self._check(self.L.dnlo_internal_forces(self.h))
        return self.array("fint").copy()

    def prologue(self):
        self._check(self.L.dnlo_prologue(self.h))

    def steps(self, n: int) -> int:
        done = C.c_long(0)
        self._check(self.L.dnlo_steps(self.h, int(n), C.byref(done)))
        return done.value

    def courant(self) -> float:
        return self.L.dnlo_courant(self.h)

    def max_frequency(self) -> float:
        out = C.c_double(0)
        self._check(self.L.dnlo_max_frequency(self.h, C.byref(out)))
        return out.value

    def inject(self, coords, du, v, a, disp, S, Eps, EpsPlas, p, evp, dt):
        """Overwrite nodal Current fields and integration-point state (as ref_harness forces)."""
        self.array("coords")[:] = np.asarray(coords).ravel()
        self.array("du")[:] = np.asarray(du).ravel()
        self.array("v")[:] = np.asarray(v).ravel()
        self.array("a")[:] = np.asarray(a).ravel()
        self.array("disp")[:] = np.asarray(disp).ravel()
        self.array("S")[:] = np.asarray(S).ravel()
        self.array("Eps")[:] = np.asarray(Eps).ravel()
        self.array("EpsPlas")[:] = np.asarray(EpsPlas).ravel()
        self.array("p")[:] = np.asarray(p).ravel()
        self.array("evp")[:] = np.asarray(evp).ravel()
        self.set("dt", dt)


def sens_lib():
    global _sens
    if _sens is None:
        build()
        L = C.CDLL(SENS_PATH)
        dp, lp = C.POINTER(C.c_double), C.POINTER(C.c_long)
        L.dnls_create.restype = C.c_void_p
        L.dnls_create.argtypes = [C.c_int, C.c_long, C.c_long, dp, lp, dp, dp, dp, C.c_long, lp, dp,
                                  lp, lp, C.c_double]
        L.dnls_destroy.argtypes = [C.c_void_p]
        L.dnls_run.argtypes = [C.c_void_p, C.c_long, dp]
        L.dnls_coords.argtypes = [C.c_void_p, dp, dp]
        L.dnls_set_hourglass.argtypes = [C.c_void_p, C.c_double]
        _sens = L
    return _sens


def _bc_arrays(m):
    kinds = np.array([g.kind for g in m.bcs] or [0], dtype=np.int64)
    vals = np.array([list(g.val) for g in m.bcs] or [[0, 0, 0]], dtype=np.float64).ravel()
    starts = np.zeros(len(m.bcs) + 1, dtype=np.int64)
    for i, g in enumerate(m.bcs):
        starts[i + 1] = starts[i] + len(g.nodes)
    nodes = np.concatenate([np.asarray(g.nodes, dtype=np.int64) for g in m.bcs]) if m.bcs \
        else np.zeros(1, dtype=np.int64)
    return kinds, vals, starts, nodes


PARAMS = ("A", "B", "n", "v0")


class SensOracle:
    """Forward-mode sensitivities on the CPU (oracle/dnl_sens.cc): a run with a prescribed
    step-size schedule, carrying d/dp for p = (A, B, n, |v0|) in FP64 dual numbers."""

    def __init__(self, model, mass=None, threads: int = 0):
        L = sens_lib()
        if threads:
            lib().dnlo_set_threads(int(threads))
        m = model
        if mass is None:
            o = Oracle(m)
            o.prologue()
            mass = o.array("mass").copy()
        coords = np.ascontiguousarray(m.coords, dtype=np.float64)
        conn = np.ascontiguousarray(m.conn, dtype=np.int64)
        mat = np.array([m.young, m.poisson, m.density, m.A, m.B, m.n], dtype=np.float64)
        v0 = np.array(m.v0, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        kinds, vals, starts, nodes = _bc_arrays(m)
        self._keep = (coords, conn, mat, v0, mass, kinds, vals, starts, nodes)
        self.h = L.dnls_create(m.etype, m.N, m.E, _dp(coords), _lp(conn), _dp(mat), _dp(v0),
                               _dp(mass), len(m.bcs), _lp(kinds), _dp(vals), _lp(starts),
                               _lp(nodes), float(m.rho_b))
        if not self.h:
            raise ValueError("dnls_create rejected the model")
        if L.dnls_set_hourglass(self.h, float(m.hourglass)):
            raise ValueError("dnls_set_hourglass rejected the coefficient")
        self.model = m
        self.L = L

    def run(self, dts):
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        r = self.L.dnls_run(self.h, len(dts), _dp(dts))
        if r:
            raise OracleError(r, -1)

    def coords(self):
        """(coords (N, 3), d coords / dp (4, N, 3))"""
        m = self.model
        x = np.zeros((m.N, 3))
        dx = np.zeros((4, m.N, 3))
        self.L.dnls_coords(self.h, _dp(x), _dp(dx))
        return x, dx

    def __del__(self):
        if getattr(self, "h", None):
            self.L.dnls_destroy(self.h)
            self.h = None
