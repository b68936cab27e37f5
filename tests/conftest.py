import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300) and the built libarlgpu.so')


@pytest.fixture(scope='session')
def arl():
    return importlib.import_module('algorithm-reference-library_gb300')


@pytest.fixture(scope='session')
def oracle():
    from oracle import arl_oracle
    return arl_oracle


@pytest.fixture(scope='session')
def golden():
    import numpy

    def load(name):
        return numpy.load(os.path.join(GOLDEN, name))
    return load
