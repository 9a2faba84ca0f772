import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def cuda_available() -> bool:
    try:
        from redynela_gb300 import dynela
        return dynela.device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree; GPU tests fail (not skip) when it cannot be used."""
    from redynela_gb300 import build, dynela
    build.build()
    assert dynela.device_count() > 0, "no CUDA device visible to libdnlgpu"
    return dynela


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
