import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def built_lib():
    from breseq_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    return ob.build()
