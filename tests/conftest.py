import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def golden_units():
    import numpy
    return dict(numpy.load(os.path.join(REPO, 'tests', 'golden', 'reference_units.npz')))


@pytest.fixture(scope="session")
def golden_runs():
    import numpy
    return dict(numpy.load(os.path.join(REPO, 'tests', 'golden', 'reference_runs.npz')))
