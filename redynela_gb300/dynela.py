"""Python binding of libdnlgpu (include/dnl_gpu.h) over ctypes.

Two layers:

* :class:`GpuDomain` -- one handle of the C ABI for a :class:`redynela_gb300.meshes.Model`:
  ``internal_forces`` (the ``Domain::computeInternalForces`` drop-in), ``step`` / ``run`` /
  ``step_graph`` (``ExplicitSolverCH::solve`` on the device), state get/set.
* :class:`Structure` and friends -- the calls a DynELA ``.dyn`` deck makes
  (``Structure::createNode``, ``createElement``, ``attachInitialBC``, ``attachConstantBC``,
  ``ExplicitSolverCH::setTimes`` ..., see Samples/Taylor/Taylor_Axi_Parametric.dyn), building the
  same model and solving it on the GPU.

The library must be built (``python -m redynela_gb300.build``); there is no CPU fallback: a
missing library or CUDA device raises.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import meshes
from .meshes import BCGroup, Model

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libdnlgpu.so")

DNL_OK = 0
STATUS_NAMES = {
    1: "DNL_ERR_NEG_DETJ", 2: "DNL_ERR_RR_NOCONV", 3: "DNL_ERR_JACOBI_NOCONV",
    4: "DNL_ERR_PULSE_NOCONV", 5: "DNL_ERR_DT", 6: "DNL_ERR_ARG", 7: "DNL_ERR_CUDA",
    8: "DNL_ERR_SINGULAR", 9: "DNL_ERR_TIMEOUT",
}
FLAG_STEP_TENSORS = 1
PROF_KINDS = ("elem", "node", "pulse", "courant", "other", "tangent")


class DnlError(RuntimeError):
    def __init__(self, code: int, msg: str, element: int = -1):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}"
                         + (f" (element {element})" if element >= 0 else ""))
        self.code = code
        self.element = element


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class MeshDesc(C.Structure):
    _fields_ = [("etype", C.c_int), ("num_nodes", C.c_int), ("num_elements", C.c_int),
                ("coords", _dp), ("conn", _ip), ("v0", C.c_double * 3), ("num_bc", C.c_int),
                ("bc_kind", _ip), ("bc_val", _dp), ("bc_start", _ip), ("bc_nodes", _ip)]


class MaterialDesc(C.Structure):
    _fields_ = [("young", C.c_double), ("poisson", C.c_double), ("density", C.c_double),
                ("A", C.c_double), ("B", C.c_double), ("n", C.c_double)]


class MaterialLawDesc(C.Structure):
    _fields_ = [("young", C.c_double), ("poisson", C.c_double), ("density", C.c_double),
                ("law", C.c_int), ("params", C.c_double * 8), ("npoints", C.c_int),
                ("table_x", C.POINTER(C.c_double)), ("table_y", C.POINTER(C.c_double))]


class SolverParams(C.Structure):
    _fields_ = [("end_time", C.c_double), ("rho_b", C.c_double), ("safety", C.c_double),
                ("frequency", C.c_int), ("method", C.c_int), ("flags", C.c_int)]


class StateView(C.Structure):
    _fields_ = [(n, _dp) for n in ("coords", "du", "v", "a", "disp", "S", "Eps", "EpsPlas", "p",
                                   "evp", "Sig", "mass")]


class AdjointInfo(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("stride", C.c_int), ("checkpoints", C.c_int),
                ("recomputed_steps", C.c_longlong), ("bytes", C.c_longlong),
                ("checkpoint_bytes", C.c_longlong), ("record_bytes", C.c_longlong),
                ("kept_record_bytes", C.c_longlong)]


class TimeInfo(C.Structure):
    _fields_ = [("time", C.c_double), ("time_step", C.c_double), ("computed_step", C.c_double),
                ("kinetic", C.c_double), ("increment", C.c_longlong), ("done", C.c_int),
                ("status", C.c_int), ("bad_element", C.c_int)]


_lib = None


def lib():
    """Load libdnlgpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not found: run `python -m redynela_gb300.build`")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.dnl_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(MaterialDesc),
                                 C.POINTER(SolverParams), C.POINTER(H)]
        L.dnl_destroy.argtypes = [H]
        L.dnl_set_hourglass.argtypes = [H, C.c_double]
        L.dnl_add_elements.argtypes = [H, C.c_int, C.c_int, _ip]
        L.dnl_set_state.argtypes = [H, C.POINTER(StateView)]
        L.dnl_get_state.argtypes = [H, C.POINTER(StateView)]
        L.dnl_get_step_tensors.argtypes = [H, _dp, _dp]
        L.dnl_internal_forces.argtypes = [H, _dp, _dp, C.c_double, _dp]
        L.dnl_prologue.argtypes = [H]
        L.dnl_step.argtypes = [H, C.c_int, _ip]
        L.dnl_run.argtypes = [H, _ip]
        L.dnl_step_host.argtypes = [H, C.POINTER(StateView), C.c_int, C.POINTER(StateView), _ip]
        L.dnl_step_graph.argtypes = [H, C.c_int, _ip]
        L.dnl_time_step.argtypes = [H, _dp]
        L.dnl_get_time_info.argtypes = [H, C.POINTER(TimeInfo)]
        L.dnl_get_fint.argtypes = [H, _dp]
        L.dnl_error_string.restype = C.c_char_p
        L.dnl_error_string.argtypes = [C.c_int]
        L.dnl_device_count.argtypes = [_ip]
        L.dnl_kernel_launches.restype = C.c_longlong
        L.dnl_profile_begin.argtypes = [H]
        L.dnl_profile_end.argtypes = [H, _dp, C.POINTER(C.c_longlong)]
        L.dnl_get_stream.argtypes = [H, C.POINTER(C.c_void_p)]
        L.dnl_timer_mark.argtypes = [H, C.c_int]
        L.dnl_timer_elapsed.argtypes = [H, C.c_int, C.c_int, _dp]
        L.dnl_measure_fp64_peak.argtypes = [_dp]
        L.dnl_check_quotients.argtypes = [C.c_int, _dp, _dp, _dp]
        L.dnl_set_adjoint_record_budget.argtypes = [C.c_ulonglong]
        L.dnl_set_stop_tolerances.argtypes = [C.c_double, C.c_double]
        L.dnl_set_iteration_caps.argtypes = [C.c_int, C.c_int, C.c_int]
        L.dnl_set_device.argtypes = [C.c_int]
        L.dnl_host_alloc.argtypes = [C.c_ulonglong, C.POINTER(C.c_void_p)]
        L.dnl_host_free.argtypes = [C.c_void_p]
        L.dnl_range_push.argtypes = [C.c_char_p]
        L.dnl_batch_create.argtypes = [C.c_int, C.POINTER(MeshDesc), C.POINTER(MaterialDesc),
                                       C.POINTER(SolverParams), C.POINTER(H)]
        L.dnl_batch_destroy.argtypes = [H]
        L.dnl_batch_prologue.argtypes = [H]
        L.dnl_batch_step.argtypes = [H, C.c_int, _ip]
        L.dnl_batch_broadcast_state.argtypes = [H, H]
        L.dnl_batch_set_mode.argtypes = [H, C.c_int]
        L.dnl_batch_get_tuning.argtypes = [H, _ip, _ip]
        L.dnl_batch_step_graph.argtypes = [H, C.c_int, _ip]
        L.dnl_batch_graph_capture.argtypes = [H, C.c_int]
        L.dnl_batch_autotune.argtypes = [H, C.c_int, _ip]
        L.dnl_batch_set_block.argtypes = [H, C.c_int]
        L.dnl_batch_time_info.argtypes = [H, C.c_int, C.POINTER(TimeInfo)]
        L.dnl_batch_get_coords.argtypes = [H, C.c_int, _dp]
        L.dnl_batch_get_fint.argtypes = [H, C.c_int, _dp]
        L.dnl_batch_sizes.argtypes = [H, _ip, _ip]
        L.dnl_batch_handle.argtypes = [H, C.POINTER(H)]
        L.dnl_sens_run.argtypes = [H, C.c_int, _dp, _dp, _dp]
        L.dnl_set_dt_schedule.argtypes = [H, _dp, C.c_int]
        L.dnl_adjoint.argtypes = [H, _dp, _dp, C.c_int]
        L.dnl_adjoint_stats.argtypes = [H, C.POINTER(AdjointInfo)]
        L.dnl_adjoint_forward.argtypes = [H, C.c_int, _dp]
        L.dnl_adjoint_backward.argtypes = [H, _dp, _dp]
        L.dnl_run_schedule.argtypes = [H, C.c_int, _dp, _dp]
        L.dnl_reset.argtypes = [H, C.POINTER(MaterialDesc), _dp]
        L.dnl_set_materials.argtypes = [H, C.c_int, C.POINTER(MaterialLawDesc), _ip]
        L.dnl_write_results.argtypes = [H, C.c_char_p]
        L.dnl_read_results.argtypes = [H, C.c_char_p]
        L.dnl_batch_sens_run.argtypes = [H, C.c_int, _dp, _dp, _dp]
        L.dnl_batch_reset.argtypes = [H]
        _lib = L
    return _lib


def device_count() -> int:
    n = C.c_int(0)
    lib().dnl_device_count(C.byref(n))
    return n.value


def kernel_launches() -> int:
    return int(lib().dnl_kernel_launches())


def set_device(device: int) -> None:
    rc = lib().dnl_set_device(int(device))
    if rc:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())


def range_push(name: str) -> None:
    lib().dnl_range_push(name.encode())


def range_pop() -> None:
    lib().dnl_range_pop()


def set_iteration_caps(rotations: int = -1, newton: int = -1, power: int = -1) -> None:
    """dnl_set_iteration_caps: limits of the Jacobi passes, the radial return's Newton iterations
    and the Pulse power iteration (-1: the reference's 29, 2000, 1000)."""
    rc = lib().dnl_set_iteration_caps(int(rotations), int(newton), int(power))
    if rc != DNL_OK:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())


def check_quotients(a: np.ndarray, b: np.ndarray) -> Dict[str, np.ndarray]:
    """dnl_check_quotients: the kernels' Newton-Raphson reciprocal and quotient of a / b next to
    CUDA's IEEE 1 / b and a / b, computed on the current device."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.size
    out = np.zeros(4 * n)
    rc = lib().dnl_check_quotients(n, _ptr(a), _ptr(b), _ptr(out))
    if rc != DNL_OK:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())
    o = out.reshape(4, n)
    return {"rcp": o[0], "quot": o[1], "ieee_rcp": o[2], "ieee_quot": o[3]}


def set_stop_tolerances(polar: float = -1.0, radial: float = -1.0) -> None:
    """dnl_set_stop_tolerances: the polar decomposition's and the radial return's stopping
    tolerances (negative: the reference's 1e-9 and 1e-8), for derivative checks against
    difference quotients."""
    rc = lib().dnl_set_stop_tolerances(float(polar), float(radial))
    if rc:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())


def set_adjoint_record_budget(nbytes: int) -> None:
    """dnl_set_adjoint_record_budget: device bytes a reverse sweep may keep for one segment's
    per-point records (0: regenerate each by running the element pass again)."""
    rc = lib().dnl_set_adjoint_record_budget(int(nbytes))
    if rc != DNL_OK:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())


def fp64_peak_tflops() -> float:
    t = C.c_double(0)
    rc = lib().dnl_measure_fp64_peak(C.byref(t))
    if rc:
        raise DnlError(rc, lib().dnl_error_string(rc).decode())
    return t.value


class PinnedArray:
    """A float64 numpy array in page-locked host memory (dnl_host_alloc)."""

    def __init__(self, shape):
        n = int(np.prod(shape))
        p = C.c_void_p()
        rc = lib().dnl_host_alloc(8 * max(n, 1), C.byref(p))
        if rc:
            raise DnlError(rc, lib().dnl_error_string(rc).decode())
        self._p = p
        buf = (C.c_double * max(n, 1)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape)

    def __del__(self):
        if getattr(self, "_p", None) and self._p.value:
            lib().dnl_host_free(self._p)
            self._p = None


def _ptr(a: Optional[np.ndarray]):
    return a.ctypes.data_as(_dp) if a is not None else None


class GpuDomain:
    """One mesh on the GPU (a ``dnl_handle``)."""

    def __init__(self, model: Model, flags: int = 0):
        L = lib()
        if device_count() < 1:
            raise RuntimeError("libdnlgpu: no CUDA device")
        m = model
        self.model = m
        self._coords = np.ascontiguousarray(m.coords, dtype=np.float64)
        self._conn = np.ascontiguousarray(m.conn, dtype=np.int32)
        kinds = np.array([g.kind for g in m.bcs] or [0], dtype=np.int32)
        vals = np.array([list(g.val) for g in m.bcs] or [[0.0, 0.0, 0.0]], dtype=np.float64)
        starts = np.zeros(len(m.bcs) + 1, dtype=np.int32)
        for i, g in enumerate(m.bcs):
            starts[i + 1] = starts[i] + len(g.nodes)
        nodes = (np.concatenate([np.asarray(g.nodes) for g in m.bcs]).astype(np.int32)
                 if m.bcs else np.zeros(1, dtype=np.int32))
        self._bc = (kinds, vals, starts, nodes)
        desc = MeshDesc(m.etype, m.N, m.E, self._coords.ctypes.data_as(_dp),
                        self._conn.ctypes.data_as(_ip), (C.c_double * 3)(*m.v0), len(m.bcs),
                        kinds.ctypes.data_as(_ip), vals.ctypes.data_as(_dp),
                        starts.ctypes.data_as(_ip), nodes.ctypes.data_as(_ip))
        mat = MaterialDesc(m.young, m.poisson, m.density, m.A, m.B, m.n)
        sp = SolverParams(m.tend, m.rho_b, m.safety, int(m.freq), int(m.method), int(flags))
        h = C.c_void_p()
        self._check(L.dnl_create(C.byref(desc), C.byref(mat), C.byref(sp), C.byref(h)))
        self.h = h
        self.L = L
        # further element groups first: the materials then cover every group's elements
        self._groups = []
        for etype, conn in (m.groups or []):
            self.add_elements(etype, conn)
        if m.materials or m.elem_material is not None:
            self.set_materials(m.material_laws(), m.elem_material)
        if m.initial_velocity is not None:
            self.set_state(v=np.asarray(m.initial_velocity, dtype=np.float64))
        if m.etype == meshes.ELHEX8N3D_1PT:
            self.set_hourglass(m.hourglass)

    def add_elements(self, etype: int, conn) -> None:
        """dnl_add_elements: a further group of elements of another type in this domain, numbered
        after the elements already there (before the prologue)."""
        c = np.ascontiguousarray(conn, dtype=np.int32)
        self._check(self.L.dnl_add_elements(self.h, int(etype), int(c.shape[0]), c.ctypes.data_as(_ip)))
        self._groups.append(c)

    def set_hourglass(self, coefficient: float) -> None:
        """dnl_set_hourglass: the one-point hexahedron's viscous hourglass coefficient."""
        self._check(self.L.dnl_set_hourglass(self.h, float(coefficient)))

    def set_materials(self, laws, elem_material=None) -> None:
        """dnl_set_materials: materials with their hardening laws, one per element."""
        arr = (MaterialLawDesc * len(laws))()
        keep = []
        for i, ml in enumerate(laws):
            prm = list(ml.params) + [0.0] * (8 - len(ml.params))
            tx = np.ascontiguousarray(ml.table_x if ml.table_x is not None else np.zeros(1), dtype=np.float64)
            ty = np.ascontiguousarray(ml.table_y if ml.table_y is not None else np.zeros(1), dtype=np.float64)
            keep += [tx, ty]
            npts = len(ml.table_x) if ml.table_x is not None else 0
            arr[i] = MaterialLawDesc(ml.young, ml.poisson, ml.density, int(ml.law), (C.c_double * 8)(*prm),
                                     npts, tx.ctypes.data_as(_dp), ty.ctypes.data_as(_dp))
        em = None if elem_material is None else np.ascontiguousarray(elem_material, dtype=np.int32)
        nel = self.model.E + sum(c.shape[0] for c in getattr(self, "_groups", []))
        if em is not None and em.size != nel:  # the library reads one index per element
            raise ValueError(f"set_materials: {em.size} element materials for {nel} elements")
        self._check(self.L.dnl_set_materials(self.h, len(laws), arr,
                                             em.ctypes.data_as(_ip) if em is not None else None))

    def close(self):
        if getattr(self, "h", None):
            self.L.dnl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, element: int = -1):
        if rc != DNL_OK:
            raise DnlError(rc, lib().dnl_error_string(rc).decode(), element)

    def _check_run(self, rc: int):
        if rc != DNL_OK:
            info = self.time_info() if rc not in (6, 7) else None
            self._check(rc, info["bad_element"] if info else -1)

    # ------------------------------------------------------------------ state
    @property
    def nip(self) -> int:
        return self.model.nip

    def _state_shapes(self) -> Dict[str, tuple]:
        """Nodal fields (N, 3); integration-point fields (E, nip, ...) with one element type, or
        (nIP, ...) over every group in element order with several."""
        m = self.model
        ip = (m.nIP_all,) if m.groups else (m.E, m.nip)
        return {"coords": (m.N, 3), "du": (m.N, 3), "v": (m.N, 3), "a": (m.N, 3),
                "disp": (m.N, 3), "S": ip + (3, 3), "Eps": ip + (3, 3),
                "EpsPlas": ip + (3, 3), "Sig": ip + (3, 3), "p": ip,
                "evp": ip, "mass": (m.N,)}

    def set_state(self, **arrays) -> None:
        """dnl_set_state; each array must hold as many values as its field (_state_shapes): the
        library reads that many."""
        shapes = self._state_shapes()
        keep = {}
        sv = StateView()
        for k, v in arrays.items():
            if v is None:
                continue
            a = np.ascontiguousarray(v, dtype=np.float64)
            if k not in shapes or k in ("Sig", "mass") or a.size != int(np.prod(shapes[k])):
                raise ValueError(f"set_state: {k} must be a writable field of {shapes.get(k)} values")
            keep[k] = a
            setattr(sv, k, a.ctypes.data_as(_dp))
        self._check(self.L.dnl_set_state(self.h, C.byref(sv)))

    def get_state(self, *names: str) -> Dict[str, np.ndarray]:
        """Nodal fields (N, 3); integration-point fields (E, nip, ...) with one element type, or
        (nIP, ...) over every group in element order with several."""
        shapes = self._state_shapes()
        names = names or tuple(shapes)
        out = {n: np.zeros(shapes[n]) for n in names}
        sv = StateView()
        for n, a in out.items():
            setattr(sv, n, a.ctypes.data_as(_dp))
        self._check(self.L.dnl_get_state(self.h, C.byref(sv)))
        return out

    def step_tensors(self):
        """dEps and R of the last element pass, shaped as the integration-point tensors."""
        shape = self._state_shapes()["S"]
        dE = np.zeros(shape)
        R = np.zeros(shape)
        self._check(self.L.dnl_get_step_tensors(self.h, _ptr(dE), _ptr(R)))
        return dE, R

    def fint(self) -> np.ndarray:
        out = np.zeros(self.model.N * self.model.dim)
        self._check(self.L.dnl_get_fint(self.h, _ptr(out)))
        return out

    # ------------------------------------------------------------------ compute
    def internal_forces(self, coords=None, du=None, dt: float = 0.0) -> np.ndarray:
        """Domain::computeInternalForces drop-in; returns Fint (dim*N, index Id*dim+j)."""
        c = np.ascontiguousarray(coords, dtype=np.float64) if coords is not None else None
        d = np.ascontiguousarray(du, dtype=np.float64) if du is not None else None
        out = np.zeros(self.model.N * self.model.dim)
        self._check_run(self.L.dnl_internal_forces(self.h, _ptr(c), _ptr(d), float(dt), _ptr(out)))
        return out

    def prologue(self) -> None:
        self._check_run(self.L.dnl_prologue(self.h))

    def step(self, n: int = 1) -> int:
        done = C.c_int(0)
        self._check_run(self.L.dnl_step(self.h, int(n), C.byref(done)))
        return done.value

    def step_graph(self, n: int) -> int:
        done = C.c_int(0)
        self._check_run(self.L.dnl_step_graph(self.h, int(n), C.byref(done)))
        return done.value

    NODAL = ("coords", "du", "v", "a", "disp")

    def step_host(self, n: int = 1, inputs: Optional[Dict[str, np.ndarray]] = None,
                  outputs: Optional[Dict[str, np.ndarray]] = None) -> int:
        """dnl_step_host: upload the nodal fields of ``inputs`` ((N, 3) each), run n steps and
        download into the arrays of ``outputs`` ((N, 3) float64, C-contiguous, written in place;
        page-locked arrays such as PinnedArray keep the copies asynchronous).  The same results as
        set_state + step + get_state."""
        shape = (self.model.N, 3)
        views, keep = [], []
        for fields, writable in ((inputs, False), (outputs, True)):
            if fields is None:
                views.append(None)
                continue
            sv = StateView()
            for k, v in fields.items():
                if k not in self.NODAL:
                    raise ValueError(f"step_host: {k} is not a nodal field")
                a = v if writable else np.ascontiguousarray(v, dtype=np.float64)
                if a.dtype != np.float64 or a.shape != shape or not a.flags.c_contiguous:
                    raise ValueError(f"step_host: {k} must be a C-contiguous float64 array {shape}")
                keep.append(a)
                setattr(sv, k, a.ctypes.data_as(_dp))
            views.append(sv)
        done = C.c_int(0)
        self._check_run(self.L.dnl_step_host(self.h, C.byref(views[0]) if views[0] else None, int(n),
                                             C.byref(views[1]) if views[1] else None, C.byref(done)))
        return done.value

    def run(self) -> int:
        done = C.c_int(0)
        self._check_run(self.L.dnl_run(self.h, C.byref(done)))
        return done.value

    def time_step(self) -> float:
        dt = C.c_double(0)
        self._check(self.L.dnl_time_step(self.h, C.byref(dt)))
        return dt.value

    def profile_begin(self) -> None:
        self._check(self.L.dnl_profile_begin(self.h))

    def profile_end(self) -> Dict[str, tuple]:
        """{kernel class: (milliseconds, launches)} since profile_begin."""
        ms = np.zeros(len(PROF_KINDS))
        n = (C.c_longlong * len(PROF_KINDS))()
        self._check(self.L.dnl_profile_end(self.h, _ptr(ms), n))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(PROF_KINDS)}

    def timer_mark(self, slot: int) -> None:
        self._check(self.L.dnl_timer_mark(self.h, int(slot)))

    def timer_elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double(0)
        self._check(self.L.dnl_timer_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        """The handle's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = C.c_void_p()
        self._check(self.L.dnl_get_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def time_info(self) -> dict:
        t = TimeInfo()
        self._check(self.L.dnl_get_time_info(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in TimeInfo._fields_}

    def reset(self, model: Optional[Model] = None) -> None:
        """dnl_reset: back to the initial state; with ``model`` (same mesh), take its material and
        initial velocity."""
        if model is None:
            self._check(self.L.dnl_reset(self.h, None, None))
            return
        mat = MaterialDesc(model.young, model.poisson, model.density, model.A, model.B, model.n)
        v0 = np.ascontiguousarray(model.v0, dtype=np.float64)
        self._check(self.L.dnl_reset(self.h, C.byref(mat), _ptr(v0)))
        self.model = model

    def write_results(self, path: str) -> None:
        """dnl_write_results: the reference's binary results file (needs FLAG_STEP_TENSORS)."""
        self._check(self.L.dnl_write_results(self.h, os.fsencode(path)))

    def read_results(self, path: str) -> None:
        """dnl_read_results: load a results file of this mesh and continue from its time."""
        self._check_run(self.L.dnl_read_results(self.h, os.fsencode(path)))

    def sensitivities(self, dts):
        """dnl_sens_run: the run with step sizes ``dts`` from the initial state; returns the final
        coordinates (N, 3) and their derivatives (4, N, 3) with respect to SENS_PARAMS."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        N = self.model.N
        x = np.zeros((N, 3))
        dx = np.zeros((SENS_NPARAM, N, 3))
        self._check_run(self.L.dnl_sens_run(self.h, len(dts), _ptr(dts), _ptr(x), _ptr(dx)))
        return x, dx

    def adjoint(self, dL_dx, dts, ckpt_stride: int = 0) -> np.ndarray:
        """dnl_set_dt_schedule + dnl_adjoint: the reverse-mode gradient of L(x_final) with respect to
        SENS_PARAMS given dL/dx_final (N, 3), from the handle's initial state, checkpoints every
        ``ckpt_stride`` steps (0: ceil(sqrt(steps))).  The handle is at its initial state after."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        g = np.ascontiguousarray(dL_dx, dtype=np.float64)
        assert g.size == 3 * self.model.N
        self._check(self.L.dnl_set_dt_schedule(self.h, _ptr(dts), len(dts)))
        grad = np.zeros(SENS_NPARAM)
        self._check_run(self.L.dnl_adjoint(self.h, _ptr(g), _ptr(grad), int(ckpt_stride)))
        return grad

    def adjoint_forward(self, dts, ckpt_stride: int = 0) -> np.ndarray:
        """dnl_set_dt_schedule + dnl_adjoint_forward: the scheduled run from the initial state with
        its checkpoints; returns the final coordinates (N, 3)."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        self._check(self.L.dnl_set_dt_schedule(self.h, _ptr(dts), len(dts)))
        x = np.zeros((self.model.N, 3))
        self._check_run(self.L.dnl_adjoint_forward(self.h, int(ckpt_stride), _ptr(x)))
        return x

    def adjoint_backward(self, dL_dx) -> np.ndarray:
        """dnl_adjoint_backward: the reverse sweep over the last forward sweep's checkpoints."""
        g = np.ascontiguousarray(dL_dx, dtype=np.float64)
        assert g.size == 3 * self.model.N
        grad = np.zeros(SENS_NPARAM)
        self._check_run(self.L.dnl_adjoint_backward(self.h, _ptr(g), _ptr(grad)))
        return grad

    def adjoint_stats(self) -> dict:
        """dnl_adjoint_stats: checkpoints, stride, recomputed steps and device bytes of the last
        adjoint."""
        info = AdjointInfo()
        self._check(self.L.dnl_adjoint_stats(self.h, C.byref(info)))
        return {k: getattr(info, k) for k, _ in AdjointInfo._fields_}

    def run_schedule(self, dts) -> np.ndarray:
        """dnl_run_schedule: the run with step sizes ``dts`` from the initial state, no derivatives;
        returns the final coordinates (N, 3)."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        x = np.zeros((self.model.N, 3))
        self._check_run(self.L.dnl_run_schedule(self.h, len(dts), _ptr(dts), _ptr(x)))
        return x


def parse_results(path: str, num_nodes: int, num_points: int) -> Dict[str, np.ndarray]:
    """Decode a results file in the reference's binary format (see dnl_write_results): headers,
    times, per node coords ro dro e de T v a fe du disp, per integration point p evp S Sig Eps dEps
    EpsPlas (tensors (n, 3, 3)), separators."""
    d = np.fromfile(path, dtype=np.float64)
    expect = 6 + 1 + 6 + 1 + 23 * num_nodes + 3 + 47 * num_points + 3 + 3
    if d.size != expect:
        raise ValueError(f"{path}: {d.size} doubles, expected {expect}")
    out = {"header": d[0:6].copy(), "structure_time": float(d[6]), "domain_header": d[7:13].copy(),
           "time": float(d[13])}
    nodes = d[14:14 + 23 * num_nodes].reshape(num_nodes, 23)
    for name, a, b in (("coords", 0, 3), ("thermal", 3, 8), ("v", 8, 11), ("a", 11, 14),
                       ("fe", 14, 17), ("du", 17, 20), ("disp", 20, 23)):
        out[name] = nodes[:, a:b].copy()
    o = 14 + 23 * num_nodes
    out["separators"] = [d[o:o + 3].copy()]
    ips = d[o + 3:o + 3 + 47 * num_points].reshape(num_points, 47)
    out["p"], out["evp"] = ips[:, 0].copy(), ips[:, 1].copy()
    for k, name in enumerate(("S", "Sig", "Eps", "dEps", "EpsPlas")):
        out[name] = ips[:, 2 + 9 * k:11 + 9 * k].reshape(num_points, 3, 3).copy()
    o += 3 + 47 * num_points
    out["separators"] += [d[o:o + 3].copy(), d[o + 3:o + 6].copy()]
    return out


BATCH_LAUNCHES = 0
BATCH_PERSISTENT = 1

SENS_NPARAM = 4
SENS_PARAMS = ("A", "B", "n", "v0")


def model_with_params(model: Model, A: float, B: float, n: float, v0: float) -> Model:
    """The model with hardening (A, B, n) and initial-velocity magnitude v0 (direction kept)."""
    import dataclasses
    u = np.asarray(model.v0, dtype=np.float64)
    nu = float(np.linalg.norm(u))
    return dataclasses.replace(model, A=float(A), B=float(B), n=float(n),
                               v0=tuple(u / nu * float(v0)) if nu > 0 else tuple(u))


def taylor_autograd(mode: str = "reverse", ckpt_stride: int = 0):
    """torch.autograd.Function over the GPU run: forward(params, model, dts) -> final coordinates.

    ``params`` is a float64 tensor (A, B, n, |v0|).  mode "reverse": the forward pass runs the
    scheduled run with its checkpoints (dnl_adjoint_forward, ``ckpt_stride`` steps per checkpoint,
    0: ceil(sqrt(steps))) and the backward pass the reverse sweep over them
    (dnl_adjoint_backward) with the incoming gradient as dL/dx_final.  mode "forward": the forward pass runs dnl_sens_run, which returns the
    final coordinates and their derivatives, and the backward pass contracts the incoming gradient
    with those (forward-mode Jacobian)."""
    import torch

    class TaylorRun(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, model, dts):
            A, B, n, v0 = (float(v) for v in params.detach().cpu().tolist())
            d = GpuDomain(model_with_params(model, A, B, n, v0))
            if mode == "forward":
                try:
                    x, dx = d.sensitivities(dts)
                finally:
                    d.close()
                ctx.dx = torch.from_numpy(dx).to(params.device)
            else:
                x = d.adjoint_forward(dts, ckpt_stride)
                ctx.domain = d
            return torch.from_numpy(x).to(params.device)

        @staticmethod
        def backward(ctx, grad_x):
            if mode == "forward":
                dx = ctx.dx
                g = (dx * grad_x.to(dx.dtype).unsqueeze(0)).sum(dim=(1, 2))
                return g, None, None
            d = ctx.domain
            try:
                g = d.adjoint_backward(grad_x.detach().to(torch.float64).cpu().numpy())
            finally:
                d.close()
            return torch.from_numpy(g).to(grad_x.device), None, None

    return TaylorRun


class _HandleView(GpuDomain):
    """Timer/profiling access to a handle owned by someone else (a batch's union mesh)."""

    def __init__(self, h, model):  # noqa: D401 -- no dnl_create
        self.h = h
        self.L = lib()
        self.model = model

    def close(self):
        self.h = None


class BatchDomain:
    """Many meshes advanced together (dnl_batch_*)."""

    def __init__(self, models: Sequence[Model]):
        L = lib()
        if device_count() < 1:
            raise RuntimeError("libdnlgpu: no CUDA device")
        self.models = list(models)
        n = len(self.models)
        descs = (MeshDesc * n)()
        mats = (MaterialDesc * n)()
        sps = (SolverParams * n)()
        self._keep = []
        for i, m in enumerate(self.models):
            coords = np.ascontiguousarray(m.coords, dtype=np.float64)
            conn = np.ascontiguousarray(m.conn, dtype=np.int32)
            kinds = np.array([g.kind for g in m.bcs] or [0], dtype=np.int32)
            vals = np.array([list(g.val) for g in m.bcs] or [[0.0, 0.0, 0.0]], dtype=np.float64)
            starts = np.zeros(len(m.bcs) + 1, dtype=np.int32)
            for j, g in enumerate(m.bcs):
                starts[j + 1] = starts[j] + len(g.nodes)
            nodes = (np.concatenate([np.asarray(g.nodes) for g in m.bcs]).astype(np.int32)
                     if m.bcs else np.zeros(1, dtype=np.int32))
            self._keep += [coords, conn, kinds, vals, starts, nodes]
            descs[i] = MeshDesc(m.etype, m.N, m.E, coords.ctypes.data_as(_dp),
                                conn.ctypes.data_as(_ip), (C.c_double * 3)(*m.v0), len(m.bcs),
                                kinds.ctypes.data_as(_ip), vals.ctypes.data_as(_dp),
                                starts.ctypes.data_as(_ip), nodes.ctypes.data_as(_ip))
            mats[i] = MaterialDesc(m.young, m.poisson, m.density, m.A, m.B, m.n)
            sps[i] = SolverParams(m.tend, m.rho_b, m.safety, int(m.freq), int(m.method), 0)
        h = C.c_void_p()
        rc = L.dnl_batch_create(n, descs, mats, sps, C.byref(h))
        if rc:
            raise DnlError(rc, L.dnl_error_string(rc).decode())
        self.h = h
        self.L = L
        E, N = C.c_int(0), C.c_int(0)
        L.dnl_batch_sizes(h, C.byref(E), C.byref(N))
        self.E, self.N = E.value, N.value

    def close(self):
        if getattr(self, "h", None):
            self.L.dnl_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise DnlError(rc, self.L.dnl_error_string(rc).decode())

    def prologue(self):
        self._check(self.L.dnl_batch_prologue(self.h))

    def step(self, n: int) -> int:
        act = C.c_int(0)
        self._check(self.L.dnl_batch_step(self.h, int(n), C.byref(act)))
        return act.value

    def graph_capture(self, n: int) -> None:
        """dnl_batch_graph_capture: capture, without running, the graph step_graph(n) replays."""
        self._check(self.L.dnl_batch_graph_capture(self.h, int(n)))

    def step_graph(self, n: int) -> int:
        act = C.c_int(0)
        self._check(self.L.dnl_batch_step_graph(self.h, int(n), C.byref(act)))
        return act.value

    def autotune(self, steps: int = 3) -> int:
        b = C.c_int(0)
        self._check(self.L.dnl_batch_autotune(self.h, int(steps), C.byref(b)))
        return b.value

    def set_block(self, block: int):
        self._check(self.L.dnl_batch_set_block(self.h, int(block)))

    def set_mode(self, mode: int):
        """dnl_batch_set_mode: BATCH_LAUNCHES (a launch sequence per step) or BATCH_PERSISTENT
        (one persistent cooperative kernel per step)."""
        self._check(self.L.dnl_batch_set_mode(self.h, int(mode)))

    def tuning(self):
        """dnl_batch_get_tuning: (mode, block) in use."""
        mo, bl = C.c_int(0), C.c_int(0)
        self._check(self.L.dnl_batch_get_tuning(self.h, C.byref(mo), C.byref(bl)))
        return mo.value, bl.value

    def time_info(self, i: int) -> dict:
        t = TimeInfo()
        self._check(self.L.dnl_batch_time_info(self.h, int(i), C.byref(t)))
        return {k: getattr(t, k) for k, _ in TimeInfo._fields_}

    def coords(self, i: int) -> np.ndarray:
        out = np.zeros((self.models[i].N, 3))
        self._check(self.L.dnl_batch_get_coords(self.h, int(i), _ptr(out)))
        return out

    def fint(self, i: int) -> np.ndarray:
        out = np.zeros(self.models[i].N * self.models[i].dim)
        self._check(self.L.dnl_batch_get_fint(self.h, int(i), _ptr(out)))
        return out

    def reset(self) -> None:
        """dnl_batch_reset: every instance back to its initial state."""
        self._check(self.L.dnl_batch_reset(self.h))

    def broadcast_state(self, domain: "GpuDomain") -> None:
        """dnl_batch_broadcast_state: the state of a single-mesh handle (same mesh as every
        instance) copied into every instance."""
        self._check(self.L.dnl_batch_broadcast_state(self.h, domain.h))

    def sensitivities(self, dts, outputs: bool = True):
        """dnl_batch_sens_run: every instance with step sizes ``dts``; returns, per instance, the
        final coordinates (N_i, 3) and their derivatives (4, N_i, 3) (nothing if not outputs)."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        if not outputs:
            self._check(self.L.dnl_batch_sens_run(self.h, len(dts), _ptr(dts), None, None))
            return None
        x = np.zeros((self.N, 3))
        dx = np.zeros((SENS_NPARAM, self.N, 3))
        self._check(self.L.dnl_batch_sens_run(self.h, len(dts), _ptr(dts), _ptr(x), _ptr(dx)))
        out, off = [], 0
        for m in self.models:
            out.append((x[off:off + m.N].copy(), dx[:, off:off + m.N].copy()))
            off += m.N
        return out

    def handle_view(self) -> GpuDomain:
        """Timer marks / profiling on the batch's stream."""
        hh = C.c_void_p()
        self._check(self.L.dnl_batch_handle(self.h, C.byref(hh)))
        return _HandleView(hh, self.models[0])


# ====================================================================== deck-level mirror
class Material:
    """Material (finiteElement/Material.h:61-156): setYoung, setPoisson, setDensity, setHardening
    (no hardening attached: elastic)."""

    def __init__(self):
        self.young = 0.0
        self.poisson = 0.0
        self.density = 0.0
        self.hardening = None

    def setYoung(self, v):
        self.young = float(v)

    def setPoisson(self, v):
        self.poisson = float(v)

    def setDensity(self, v):
        self.density = float(v)

    def setHardening(self, h):
        self.hardening = h

    def setColor(self, r, g, b):
        pass  # post-processing colour

    def law(self) -> meshes.MaterialLaw:
        """The library's description of this material and its hardening."""
        h = self.hardening
        if h is None:
            return meshes.MaterialLaw(self.young, self.poisson, self.density, meshes.HARD_ELASTIC)
        return h._law(self)


class IsoHardElastoplastic:
    """sigma_y = A + B evp^n (finiteElement/IsoHardElastoplastic.C:171-184)."""

    def __init__(self):
        self.A = self.B = 0.0
        self.n = 1.0

    def setYieldStress(self, v):
        self.A = float(v)

    def setHardParameter(self, v):
        self.B = float(v)

    def setHardExponent(self, v):
        self.n = float(v)

    def _law(self, m: Material) -> meshes.MaterialLaw:
        return meshes.MaterialLaw(m.young, m.poisson, m.density, meshes.HARD_POWER, (self.A, self.B, self.n))


class DiscreteFunction:
    """DiscreteFunction (basicTools/DiscreteFunction.C): points (x, y) kept sorted by x."""

    def __init__(self):
        self.points: List[tuple] = []

    def add(self, x, y):
        self.points.append((float(x), float(y)))
        self.points.sort(key=lambda q: q[0])


class IsoHardElastoplasticTabular:
    """sigma_y tabulated against evp by a DiscreteFunction
    (finiteElement/IsoHardElastoplasticTabular.C:103-116)."""

    def __init__(self):
        self.function = None

    def setFunction(self, f: DiscreteFunction):
        self.function = f

    def _law(self, m: Material) -> meshes.MaterialLaw:
        xs = np.array([q[0] for q in self.function.points])
        ys = np.array([q[1] for q in self.function.points])
        return meshes.MaterialLaw(m.young, m.poisson, m.density, meshes.HARD_TABULAR, (), xs, ys)


class IsoHardMetafor:
    """sigma_y = (P2 - P1)(1 - exp(-P3 evp)) + P4 evp^P5 + P1 (1 + P6 evp)^P7 + P8 evp
    (finiteElement/IsoHardMetafor.C:132-153); set(k, value) is getConstitutiveParameter(k) = value."""

    def __init__(self):
        self.P = [0.0] * 8

    def set(self, k, v):
        self.P[int(k)] = float(v)

    def _law(self, m: Material) -> meshes.MaterialLaw:
        return meshes.MaterialLaw(m.young, m.poisson, m.density, meshes.HARD_METAFOR, tuple(self.P))


class NodeSet:
    def __init__(self):
        self.numbers: List[int] = []

    def add(self, start, stop=None, inc=1):
        """NodeSet::add(num) or add(start, stop, inc) with 1-based inclusive numbers."""
        if stop is None:
            self.numbers.append(int(start))
        else:
            self.numbers.extend(range(int(start), int(stop) + 1, int(inc)))


class ElementSet(NodeSet):
    pass


class BoundarySpeed:
    def __init__(self):
        self.val = (0.0, 0.0, 0.0)

    def set(self, x, y, z):
        self.val = (float(x), float(y), float(z))


class BoundaryRestrain(BoundarySpeed):
    pass


class ExplicitSolverCH:
    """ExplicitSolverCH settings (finiteElement/ExplicitSolverCH.C, Solver.C)."""

    def __init__(self):
        self.start, self.end = 0.0, 0.0
        self.rho_b = 0.8182
        self.safety = 0.9
        self.frequency = 10
        self.method = meshes.PULSE  # the ExplicitSolverCH constructor's default

    def setTimes(self, start, stop):
        self.start, self.end = float(start), float(stop)

    def setDissipation(self, v):
        if not 0.0 <= v <= 1.0:
            raise ValueError("dissipation value out of range [0.0, 1.0]")
        self.rho_b = float(v)

    def setTimeStepSafetyFactor(self, v):
        self.safety = float(v)

    def setComputeTimeStepFrequency(self, v):
        self.frequency = int(v)

    def setTimeStepMethod(self, name):
        """Solver::setTimeStepMethod (Solver.C:312-322): "Courant" or "Pulse"."""
        if name not in ("Courant", "Pulse"):
            raise ValueError(f"setTimeStepMethod: unknown method {name}")
        self.method = {"Courant": meshes.COURANT, "Pulse": meshes.PULSE}[name]


ElQua4nAx = meshes.ELQUA4NAX
ElHex8n3D = meshes.ELHEX8N3D
ElQua4n2D = meshes.ELQUA4N2D
ElTet4n3D = meshes.ELTET4N3D
ElTet10n3D = meshes.ELTET10N3D
ElHex8n3D_1PT = meshes.ELHEX8N3D_1PT


class Structure:
    """The model-building calls of a .dyn deck (finiteElement/Structure.h), solved on the GPU.

    Elements are numbered in creation order (Structure::createElement); a setDefaultElement of
    another type between createElement calls starts a further element group (3D reference
    elements; dnl_add_elements).  Each attachMaterialToElements sets the material of its set's
    elements (later attachments win), each attachInitialBC the initial velocity of its set's
    nodes (BoundarySpeed::applyInitial_V0), each attachConstantBC a restraint (BoundaryRestrain) or
    an imposed speed (BoundarySpeed) on its set's nodes."""

    def __init__(self):
        self._nodes: Dict[int, Sequence[float]] = {}
        self._elements: List[tuple] = []  # (number, etype, node numbers) in creation order
        self._etype = None
        self._materials: List[tuple] = []  # (Material, ElementSet)
        self._initial = []
        self._constant = []
        self._solver = None
        self.domain: Optional[GpuDomain] = None

    def createNode(self, num, x, y, z):
        self._nodes[int(num)] = (float(x), float(y), float(z))

    def setDefaultElement(self, etype):
        self._etype = etype

    def createElement(self, num, *nodes):
        if self._etype is None:
            raise ValueError("createElement: no default element type (setDefaultElement)")
        self._elements.append((int(num), self._etype, tuple(int(n) for n in nodes)))

    def addMaterial(self, mat):
        pass  # materials enter through attachMaterialToElements

    def attachMaterialToElements(self, mat, els):
        self._materials.append((mat, els))

    def attachInitialBC(self, bnd, nodes):
        self._initial.append((bnd, nodes))

    def attachConstantBC(self, bnd, nodes):
        self._constant.append((bnd, nodes))

    def addSolver(self, solver):
        self._solver = solver

    def setSaveTimes(self, start, stop, interval):
        pass

    def model(self) -> Model:
        nums = sorted(self._nodes)
        index = {n: i for i, n in enumerate(nums)}
        coords = np.array([self._nodes[n] for n in nums], dtype=np.float64)
        N = len(nums)
        # element groups: runs of one type in creation order
        runs: List[tuple] = []
        for num, et, nodes in self._elements:
            if not runs or runs[-1][0] != et:
                runs.append((et, []))
            runs[-1][1].append([index[n] for n in nodes])
        if not runs:
            raise ValueError("model: no elements")
        conns = [(et, np.array(c, dtype=np.int64)) for et, c in runs]
        enum = {num: i for i, (num, _, _) in enumerate(self._elements)}
        E = len(self._elements)
        # materials: each attachment sets its elements' material, later ones win
        if not self._materials:
            raise ValueError("model: no material attached")
        mats: List[Material] = []
        em = np.full(E, -1, dtype=np.int64)
        for mat, els in self._materials:
            if mat not in mats:
                mats.append(mat)
            em[[enum[n] for n in els.numbers]] = mats.index(mat)
        if np.any(em < 0):
            raise ValueError("model: elements without a material")
        used = sorted(set(em.tolist()))
        mats = [mats[i] for i in used]
        em = np.searchsorted(used, em)
        laws = [m.law() for m in mats]
        first = laws[0]
        A, B, n = (first.params if first.law == meshes.HARD_POWER else (0.0, 0.0, 1.0))
        single = len(laws) == 1 and first.law == meshes.HARD_POWER
        # initial velocities per node, later attachments win; one speed on every node is v0
        vel = np.zeros((N, 3))
        covered = np.zeros(N, dtype=bool)
        for bnd, ns in self._initial:
            idx = [index[k] for k in ns.numbers]
            vel[idx] = bnd.val
            covered[idx] = True
        uniform = bool(covered.all()) and bool(np.all(vel == vel[0])) if N else True
        v0 = tuple(vel[0]) if uniform else (0.0, 0.0, 0.0)
        bcs = []
        for bnd, ns in self._constant:
            kind = meshes.RESTRAIN if isinstance(bnd, BoundaryRestrain) else meshes.SPEED
            bcs.append(BCGroup(kind, bnd.val, np.array([index[k] for k in ns.numbers], dtype=np.int64)))
        s = self._solver
        if s is None:
            raise ValueError("model: no solver (addSolver)")
        (et0, conn0), rest = conns[0], conns[1:]
        return Model(et0, coords, conn0, first.young, first.poisson, first.density, A, B, n, v0, bcs,
                     s.end, s.rho_b, s.safety, s.frequency, s.method,
                     materials=None if single else laws, elem_material=None if single else em,
                     initial_velocity=None if uniform else vel, groups=rest or None)

    def initSolve(self, flags: int = 0) -> GpuDomain:
        self.domain = GpuDomain(self.model(), flags)
        return self.domain

    def solve(self) -> int:
        if self.domain is None:
            self.initSolve()
        return self.domain.run()
