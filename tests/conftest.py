import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library and the oracle once per session."""
    import __graft_entry__ as ge

    ge.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    import hann_gb300

    hann_gb300.load_library()
    return True
