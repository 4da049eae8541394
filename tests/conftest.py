import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # the slowest tests with their run times (the full-size configs carry
    # their nonzero count in the test id)
    if not config.option.durations:
        config.option.durations = 15


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libParTI.so and the oracle in-tree (no-op when up to date)."""
    from sptol_gb300 import build as B
    B.build()
    import oracle
    oracle.build(with_ref=False)
    yield


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def rel_fro(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return d / n if n > 0 else d


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
