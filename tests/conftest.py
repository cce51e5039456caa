import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle_binding():
    import oracle

    return oracle.binding()


@pytest.fixture(scope="session")
def gpu_binding():
    from icsfoam_gb300 import gpu

    return gpu.binding()
