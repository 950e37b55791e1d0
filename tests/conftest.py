import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def relerr(a, b):
    """Element-wise |a - b| / |b| (complex-aware), with b == 0 -> |a|."""
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.abs(a - b)
    s = np.abs(b)
    return np.where(s > 0, d / np.where(s > 0, s, 1.0), d)


@pytest.fixture(scope="session")
def golden():
    return load_golden
