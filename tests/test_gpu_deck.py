"""A deck built through the deck-level mirror (dynela.Structure) runs on the GPU as the generators'
model of the same problem, bit for bit: the Taylor deck (Structure::initSolve + the solve loop)
and the deck of a domain whose default element changes between createElement calls."""

import numpy as np
import pytest

from redynela_gb300 import meshes
from test_deck import taylor_axi_deck

pytestmark = pytest.mark.gpu


def test_taylor_deck_runs_as_the_generators_bar(gpu_lib):
    st, _ = taylor_axi_deck(5, 50)
    d = st.initSolve()
    ref = gpu_lib.GpuDomain(meshes.taylor_axi(5, 50))
    assert d.step(60) == 60 and ref.step(60) == 60
    a, b = d.get_state("coords", "v", "evp"), ref.get_state("coords", "v", "evp")
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert d.time_info() == ref.time_info()
