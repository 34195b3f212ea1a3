import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libsynk.so")


def pytest_collection_modifyitems(config, items):
    # GPU tests fail loudly when no GPU is present, unless deselected with -m "not gpu"
    pass


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("this test needs a CUDA GPU (run with -m 'not gpu' on CPU-only machines)")
    from synkrotomo_gb300 import _lib
    _lib.load(build_if_missing=True)
    return torch.device("cuda", 0)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb else 1.0))
