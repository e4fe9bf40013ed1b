import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library, built for sm_103a; GPU tests fail loudly without it."""
    import craystal_gb300
    from craystal_gb300 import build as b
    b.build()
    return craystal_gb300.load()
