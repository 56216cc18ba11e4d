import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:                 # tests/parity.py, the shared parity measures
    sys.path.insert(0, HERE)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libwotg.so')


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope='session')
def pair_golden():
    return load_golden('pair_120x150.npz')


@pytest.fixture(scope='session')
def kat_golden():
    return load_golden('kat_3x3.npz')


@pytest.fixture(scope='session')
def chain_golden():
    return load_golden('chain_maps.npz')
