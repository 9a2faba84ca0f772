"""The results-file format (the reference's Structure::writeData binary layout): the Python
decoder against the reference's own file (tests/golden/results_axi.bin, written by the compiled
reference after 13 steps of the 3x4 axisymmetric bar) and the state the harness dumped from the
same run (results_axi.npz)."""

import numpy as np
import pytest

from conftest import golden, GOLDEN
from redynela_gb300 import dynela, meshes


def test_reference_results_file_decodes_to_its_state():
    m = meshes.taylor_axi(3, 4)
    r = dynela.parse_results(f"{GOLDEN}/results_axi.bin", m.N, m.E * m.nip)
    g = golden("results_axi.npz")
    assert np.array_equal(r["header"], [3.0, 1.0, 0.0, 1.02, 0.0, 0.0])
    assert np.array_equal(r["domain_header"], r["header"])
    assert all(np.array_equal(s, [69.0, 0.0, 0.0]) for s in r["separators"])
    assert r["time"] == g["time"][-1] and r["structure_time"] == r["time"]
    for name in ("coords", "v", "a", "du", "disp"):
        assert np.array_equal(r[name].ravel(), g["final_" + name]), name
    for name in ("S", "Sig", "Eps", "dEps", "EpsPlas"):
        assert np.array_equal(r[name].ravel(), g["final_" + name]), name
    assert np.array_equal(r["p"], g["final_p"]) and np.array_equal(r["evp"], g["final_evp"])
    # after an odd number of steps the Current field is the one without the density
    assert np.all(r["thermal"] == 0.0) and np.all(r["fe"] == 0.0)


def test_truncated_file_is_rejected(tmp_path):
    m = meshes.taylor_axi(3, 4)
    data = open(f"{GOLDEN}/results_axi.bin", "rb").read()
    p = tmp_path / "short.bin"
    p.write_bytes(data[:-8])
    with pytest.raises(ValueError):
        dynela.parse_results(str(p), m.N, m.E * m.nip)
