"""pytest configuration: the `gpu` marker and session-wide builds.

Tests marked `gpu` need an sm_103 device; everything else runs on a CPU-only host
(the C-ABI library loads there and its host-side entry points work without a GPU).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) CUDA device")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the library and the oracle once (incremental; seconds when up to date)."""
    from nomad_gb300 import build as b
    from oracle import oracle as o
    b.build()
    o.build()
    yield


@pytest.fixture(scope="session")
def ng():
    import nomad_gb300
    nomad_gb300.lib()
    return nomad_gb300


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_ok(ng):
    if not ng.device_ok(0):
        pytest.fail("test marked gpu but cuda:0 is not an sm_103 device")
    return True
