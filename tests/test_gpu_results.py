"""Results / restart files on the GPU path (dnl_write_results / dnl_read_results) against the
reference's own file of the same run (tests/golden/results_axi.bin: the 3x4 axisymmetric bar after
13 steps, written by the compiled reference's Structure::writeData).  Layout, headers, separators
and the zero thermal/force fields are compared exactly; the mechanical fields to the per-step
parity tolerance (1e-12 relative 2-norm, per field)."""

import numpy as np
import pytest

from conftest import GOLDEN
from redynela_gb300 import meshes

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def test_written_file_matches_the_reference_file(gpu_lib, tmp_path):
    m = meshes.taylor_axi(3, 4)
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    assert d.step(13) == 13
    path = str(tmp_path / "gpu.bin")
    d.write_results(path)
    ours = gpu_lib.parse_results(path, m.N, m.E * m.nip)
    ref = gpu_lib.parse_results(f"{GOLDEN}/results_axi.bin", m.N, m.E * m.nip)
    for k in ("header", "domain_header"):
        assert np.array_equal(ours[k], ref[k])
    for a, b in zip(ours["separators"], ref["separators"]):
        assert np.array_equal(a, b)
    assert np.array_equal(ours["thermal"], ref["thermal"]) and np.array_equal(ours["fe"], ref["fe"])
    assert abs(ours["time"] - ref["time"]) <= 1e-15 * ref["time"]
    for k in ("coords", "v", "a", "du", "disp", "S", "Sig", "Eps", "dEps", "EpsPlas", "p", "evp"):
        assert rel(ours[k], ref[k]) <= TOL, k


def test_read_restores_the_state_and_continues(gpu_lib, tmp_path):
    """The reference's file loaded into a fresh handle gives back its state exactly; a file written
    by a handle and read into another gives the same next element pass (to the parity tolerance:
    the cached evp^n is recomputed from evp on loading), and the run continues."""
    m = meshes.taylor_axi(3, 4)
    ref = gpu_lib.parse_results(f"{GOLDEN}/results_axi.bin", m.N, m.E * m.nip)
    r = gpu_lib.GpuDomain(m)
    r.read_results(f"{GOLDEN}/results_axi.bin")
    st = r.get_state("coords", "du", "v", "a", "disp", "p", "evp")
    for k in ("coords", "du", "v", "a", "disp", "p", "evp"):
        assert np.array_equal(np.ravel(st[k]), np.ravel(ref[k])), k
    assert r.time_info()["time"] == ref["time"]
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    d.step(13)
    path = str(tmp_path / "w.bin")
    d.write_results(path)
    e = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    e.read_results(path)
    s1 = d.get_state("coords", "du", "S", "Eps", "EpsPlas", "p", "evp")
    x, du = s1["coords"], s1["du"]
    f1 = d.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    f2 = e.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    assert rel(f2, f1) <= TOL
    assert e.step(20) == 20
    assert np.all(np.isfinite(e.get_state("coords")["coords"]))


def test_writing_needs_the_step_tensors(gpu_lib, tmp_path):
    d = gpu_lib.GpuDomain(meshes.taylor_axi(3, 4))
    d.step(2)
    with pytest.raises(gpu_lib.DnlError):
        d.write_results(str(tmp_path / "x.bin"))


@pytest.mark.parametrize("model", [lambda: meshes.taylor_plane(4, 12), lambda: meshes.taylor_tet(4, 6),
                                   lambda: meshes.taylor_hex_1pt(4, 6)],
                         ids=["ElQua4n2D", "ElTet4n3D", "ElHex8n3D_1pt"])
def test_round_trip_other_elements(gpu_lib, tmp_path, model):
    """A file written by one handle and read into another, for the other element types: the nodal
    state comes back bit for bit and the next element pass agrees to the parity tolerance."""
    m = model()
    d = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    d.step(9)
    path = str(tmp_path / "w.bin")
    d.write_results(path)
    parsed = gpu_lib.parse_results(path, m.N, m.E * m.nip)
    e = gpu_lib.GpuDomain(m, flags=gpu_lib.FLAG_STEP_TENSORS)
    e.read_results(path)
    s1 = d.get_state("coords", "du", "v", "a", "disp", "p", "evp")
    s2 = e.get_state("coords", "du", "v", "a", "disp", "p", "evp")
    for k in s1:
        assert np.array_equal(np.ravel(s1[k]), np.ravel(s2[k])), k
        if k in parsed:
            assert np.array_equal(np.ravel(parsed[k]), np.ravel(s1[k])), k
    x, du = s1["coords"], s1["du"]
    f1 = d.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    f2 = e.internal_forces(coords=x, du=du, dt=d.time_info()["time_step"])
    assert rel(f2, f1) <= TOL
    assert e.step(5) == 5
