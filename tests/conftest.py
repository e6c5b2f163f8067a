"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (runs on the GB300 box)')


@pytest.fixture(scope='session', autouse=True)
def _built():
    """Build the oracle and libmcwalk in-tree if they are missing (gcc / nvcc)."""
    from oracle import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    from monte_carlompi_gb300 import build
    build.build()


def golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, '*.npz')))


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + '.npz'))


@pytest.fixture(scope='session')
def walker():
    from monte_carlompi_gb300.walker import Walker
    w = Walker(0)
    yield w
    w.close()
