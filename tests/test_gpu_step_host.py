"""dnl_step_host: steps with the nodal state exchanged with host memory in one call (v, a and disp
uploaded on a second stream beside the first element pass, the download beside the next time
step's computation) give what dnl_set_state + dnl_step + dnl_get_state give, bit for bit: every
nodal field, the time record, the integration-point state; with restrained and imposed-speed
boundary conditions (whose Current v and a writes follow the second stream's upload), the one-point
hexahedron (whose element pass reads v, uploaded first), Courant and Pulse steps, several steps per
call, a run that ends inside a call, and a domain of several element types."""

import numpy as np
import pytest

from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "du", "v", "a", "disp")


def _models():
    return {
        "axi_courant": lambda: meshes.taylor_axi(5, 50),
        "hex_pulse": lambda: meshes.taylor_hex(6, 8),
        "hex1pt": lambda: meshes.taylor_hex_1pt(6, 10),
        "necking_speed": lambda: meshes.necking_bar(4, 12, speed=5.0),
        "hex_tet": lambda: meshes.taylor_mixed(4, 8, lower=meshes.ELHEX8N3D, upper=meshes.ELTET4N3D),
    }


@pytest.mark.parametrize("kind", list(_models()))
@pytest.mark.parametrize("per_call", [1, 3])
def test_step_host_is_set_step_get(gpu_lib, kind, per_call):
    """Two handles, the same host round trip per call: A through set_state / step / get_state, B
    through step_host into page-locked arrays it reads back in place.  The host nudges the
    velocities between calls (a host-side change the next call must upload)."""
    m = _models()[kind]()
    a, b = gpu_lib.GpuDomain(m), gpu_lib.GpuDomain(m)
    a.step(4)
    b.step(4)
    host = {k: gpu_lib.PinnedArray((m.N, 3)) for k in FIELDS}
    st = b.get_state(*FIELDS)
    for k in FIELDS:
        host[k].array[:] = st[k]
    arrays = {k: host[k].array for k in FIELDS}
    for call in range(6):
        fa = a.get_state(*FIELDS)
        if call % 2:  # the host changes the velocities it owns
            fa["v"] *= 1.0 + 1e-6
            arrays["v"] *= 1.0 + 1e-6
        a.set_state(**fa)
        na = a.step(per_call)
        fa = a.get_state(*FIELDS)
        nb = b.step_host(per_call, inputs=arrays, outputs=arrays)
        assert na == nb == per_call
        for k in FIELDS:
            assert np.array_equal(arrays[k], fa[k]), (call, k)
    assert a.time_info() == b.time_info()
    sa, sb = a.get_state("S", "evp", "p"), b.get_state("S", "evp", "p")
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert np.any(sb["evp"] > 1e-10)  # plastic points


def test_step_host_partial_fields_and_early_end(gpu_lib):
    """Only coordinates in, only velocities out; then a call asking for more steps than the run has
    left stops at the end time with the fields of the last step done (the bank parity of the steps
    done, as dnl_step)."""
    m = meshes.taylor_axi(4, 30, tend=2e-6)
    a, b = gpu_lib.GpuDomain(m), gpu_lib.GpuDomain(m)
    a.step(5)
    b.step(5)
    x = a.get_state("coords")["coords"]
    x[:, 0] *= 1.0 + 1e-9
    a.set_state(coords=x)
    a.step(2)
    v = np.zeros((m.N, 3))
    assert b.step_host(2, inputs={"coords": x}, outputs={"v": v}) == 2
    assert np.array_equal(v, a.get_state("v")["v"])
    left = 10_000
    na = a.step(left)
    out = {k: np.zeros((m.N, 3)) for k in FIELDS}
    nb = b.step_host(left, outputs=out)
    assert na == nb < left and a.time_info()["done"] == b.time_info()["done"] == 1
    fa = a.get_state(*FIELDS)
    for k in FIELDS:
        assert np.array_equal(out[k], fa[k]), k


def test_step_host_refuses_integration_point_fields(gpu_lib):
    m = meshes.taylor_axi(3, 4)
    d = gpu_lib.GpuDomain(m)
    sv = gpu_lib.StateView()
    s = np.zeros(m.E * m.nip * 9)
    sv.S = s.ctypes.data_as(gpu_lib._dp)
    done = gpu_lib.C.c_int(0)
    assert gpu_lib.lib().dnl_step_host(d.h, None, 1, gpu_lib.C.byref(sv), gpu_lib.C.byref(done)) != 0
    with pytest.raises(ValueError):
        d.step_host(1, outputs={"S": s})
