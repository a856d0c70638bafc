import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs through the C-ABI library")


def golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name))


@pytest.fixture
def gold():
    return golden


@pytest.fixture
def gold_cluster():
    return golden("golden_cluster.npz")
