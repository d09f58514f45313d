import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native kernels")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2 over the grid (per component when given [g, c])."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    num = np.sqrt(np.sum((a - b) ** 2, axis=0))
    den = np.sqrt(np.sum(b ** 2, axis=0))
    return num / np.where(den > 0, den, 1.0)


def uniq(t):
    """[g, D, D] symmetric tensors -> [g, NC] unique components (xx, yy, [zz,] xy, [xz, yz])."""
    if t.shape[1] == 2:
        return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 0, 1]], axis=1)
    return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 0, 2], t[:, 1, 2]], axis=1)
