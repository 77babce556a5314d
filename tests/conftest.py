import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU; run with -m gpu")


@pytest.fixture(scope="session")
def native():
    """The product library, built in-tree if needed (fails loudly, never falls back)."""
    import starpu_gb300
    return starpu_gb300.load()


@pytest.fixture(scope="session")
def gpu(native):
    n = native.starpu_gb300_device_count()
    assert n >= 1, "GPU tests need a CUDA device: " + native.starpu_gb300_last_error().decode()
    return native


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    return O
