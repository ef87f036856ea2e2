import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Build libgfgpu.so (and the oracle) once per session."""
    from getfem_gb300 import build
    build.build()
    from oracle import gfref
    gfref.build()
    yield
