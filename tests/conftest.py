import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("jax-cpfem_gb300")


@pytest.fixture(scope="session")
def gpu(pkg):
    """(problem module, solver module) with the CUDA library loaded."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return pkg.load()
