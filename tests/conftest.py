import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
sys.path.insert(0, os.path.join(ROOT, 'tests'))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (runs on the GB300 box)')


@pytest.fixture(scope='session')
def pkg():
    import __graft_entry__ as ge
    return ge.package()


@pytest.fixture(scope='session')
def O():
    import oracle
    oracle.lib()
    return oracle
