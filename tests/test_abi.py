"""The C-ABI library: it builds for sm_103a, loads, exports every entry point include/dnl_gpu.h
declares, and rejects invalid arguments on the host.  No kernel runs here (CPU only)."""

import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "dnl_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\*?\s*\**(dnl_[a-z0-9_]+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def libpath():
    from redynela_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("dnl_create", "dnl_destroy", "dnl_internal_forces", "dnl_step", "dnl_run",
                 "dnl_get_state", "dnl_set_state", "dnl_time_step"):
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (dnl_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_reports(libpath):
    L = C.CDLL(libpath)
    L.dnl_error_string.restype = C.c_char_p
    assert L.dnl_error_string(0) == b"ok"
    assert b"Jacobian" in L.dnl_error_string(1)
    L.dnl_kernel_launches.restype = C.c_longlong
    assert L.dnl_kernel_launches() >= 0


def test_create_rejects_bad_arguments_on_host(libpath):
    """Argument checks run before any device call (usable without a GPU)."""
    from redynela_gb300 import dynela
    L = dynela.lib()
    md = dynela.MeshDesc()
    md.etype = 7
    mat = dynela.MaterialDesc(117e9, 0.35, 8930, 90e6, 292e6, 0.31)
    sp = dynela.SolverParams(80e-6, 0.8182, 0.9, 10, 0, 0)
    h = C.c_void_p()
    assert L.dnl_create(C.byref(md), C.byref(mat), C.byref(sp), C.byref(h)) == 6
    coords = np.zeros((4, 3))
    conn = np.array([0, 1, 2, 5], dtype=np.int32)  # node 5 out of range
    md = dynela.MeshDesc(0, 4, 1, coords.ctypes.data_as(dynela._dp), conn.ctypes.data_as(dynela._ip),
                         (C.c_double * 3)(0, 0, 0), 0, None, None, None, None)
    assert L.dnl_create(C.byref(md), C.byref(mat), C.byref(sp), C.byref(h)) == 6
    conn = np.array([0, 1, 2, 3], dtype=np.int32)
    md.conn = conn.ctypes.data_as(dynela._ip)
    sp_odd = dynela.SolverParams(80e-6, 0.8182, 0.9, 7, 0, 0)  # Courant with an odd frequency
    assert L.dnl_create(C.byref(md), C.byref(mat), C.byref(sp_odd), C.byref(h)) == 6
    sp_hex = dynela.SolverParams(80e-6, 0.8182, 0.9, 10, 0, 0)
    md.etype = 1  # hex8 has no Courant length (ElHex8n3D.C:188-192)
    assert L.dnl_create(C.byref(md), C.byref(mat), C.byref(sp_hex), C.byref(h)) == 6
    assert L.dnl_destroy(None) == 6


def test_host_side_refusals_of_the_newer_entry_points(libpath):
    """dnl_step_host, dnl_add_elements and dnl_set_stop_tolerances check their arguments before any
    device call: a null handle, a step count below 1, integration-point fields in a host-step view,
    tolerances of 0 or at least 1 are DNL_ERR_ARG without a GPU."""
    from redynela_gb300 import dynela
    L = dynela.lib()
    done = C.c_int(0)
    assert L.dnl_step_host(None, None, 1, None, C.byref(done)) == 6
    assert L.dnl_add_elements(None, 1, 1, None) == 6
    for polar, radial in ((0.0, 1e-8), (1e-9, 0.0), (1.0, 1e-8), (1e-9, 2.0), (float("nan"), 1e-8)):
        assert L.dnl_set_stop_tolerances(polar, radial) == 6, (polar, radial)
