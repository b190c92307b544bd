import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_vectors.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libia.so")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def cuda():
    """The GPU suite: fails (does not skip) when no GPU or no libia.so."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from inverseacoustics_gb300 import _lib
    _lib.lib()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ctx(cuda):
    from inverseacoustics_gb300 import api
    c = api.Context(0)
    yield c
    c.close()


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(np.asarray(b).ravel())
    return d / n if n > 0 else d
