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


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fpinput512():
    """The reference's dataset futhark/data/fpinputf32rad512 (the five arguments
    of forwardprojection.main) from its exact copy tests/golden/fpinputf32rad512.npz.
    A missing fixture is an error, not a skip."""
    path = os.path.join(GOLDEN, "fpinputf32rad512.npz")
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing (write it with tests/golden/make_fpinput512.py)")
    z = np.load(path)
    image = z["levels"][z["codes"]].astype(np.float32)
    return (z["angles"].astype(np.float32), np.float32(z["rhozero"]), np.float32(z["deltarho"]),
            np.int32(z["numrhos"]), image)
