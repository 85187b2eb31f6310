import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libcilgpu.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; a GPU test fails (never skips) when it is missing."""
    import cil_cuda_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        from cil_cuda_gb300 import build
        build.build()
    G.lib()
    return G
