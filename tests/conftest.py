import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    # The package refuses to import without its compiled library; build it
    # (incrementally) before collection so every test module can import it.
    from numrs_gb300 import build as b
    b.build()


@pytest.fixture(scope="session")
def ora():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def lib_path():
    from numrs_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def K(lib_path):
    """The reference-shaped host API on cuda:0 (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from numrs_gb300 import kernels
    return kernels


def to_np(t):
    return t.detach().cpu().numpy()


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view({4: np.uint32, 8: np.uint64}[a.dtype.itemsize])
