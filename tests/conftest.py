import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "triplyperiodic-modified_gb300"))
sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_err(a, b):
    """max|a-b| / max|b| (relative error of a field, as used by every parity test)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    if scale == 0:
        return float(np.abs(a).max())
    return float(np.abs(a - b).max() / scale)


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle

    pyoracle.build()
    return pyoracle
