import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def ewt():
    """The GPU library, built in-tree if needed; the tests call its C ABI."""
    import ecl_wavelet_gb300 as E
    E.build()
    E.lib()
    return E


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build_library()
    return O
