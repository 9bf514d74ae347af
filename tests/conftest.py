import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


@pytest.fixture(scope="session")
def baselines():
    """The reference's own KPM golden arrays (tests/baseline_data/kpm/*.pbz)."""
    return dict(np.load(os.path.join(GOLDEN, "kpm_baseline.npz")))


@pytest.fixture(scope="session")
def python_impl():
    """Moments computed by the reference's FP64 NumPy KPM on supplied starters."""
    return dict(np.load(os.path.join(GOLDEN, "python_impl_moments.npz")))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O
