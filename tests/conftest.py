import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on the GB300 box)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def fwn_lib():
    """The CUDA library, built in-tree if needed (fails loudly if it cannot be built)."""
    from meshlib_gb300 import build
    build.build()
    import meshlib_gb300
    return meshlib_gb300.lib()


@pytest.fixture(scope="session")
def torus():
    from meshlib_gb300 import meshgen
    return meshgen.noisy_torus(seed=1)


@pytest.fixture(scope="session")
def small_sphere():
    from meshlib_gb300 import meshgen
    return meshgen.noisy_icosphere(seed=3, level=4)  # 5,120 triangles
