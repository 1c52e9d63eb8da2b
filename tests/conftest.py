import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# f64::EPSILON
EPS = np.finfo(np.float64).eps


def equal_floats(a, b, eps=EPS):
    """test_helper::equal_floats / equal_floats_eps (src/test_helper.rs:13-40)."""
    a, b = float(a), float(b)
    if a == 0.0 and b == 0.0:
        return True
    diff = abs(a - b)
    if a == 0.0 or b == 0.0:
        return diff < eps
    return diff / min(abs(a) + abs(b), np.finfo(np.float64).max) < eps


def rel_l2(a, b):
    """Norm-wise relative error ||a - b||_2 / ||b||_2 (0 when both vanish)."""
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    na = np.linalg.norm((a - b).ravel())
    if nb == 0.0:
        return na
    return na / nb


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
