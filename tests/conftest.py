import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine64():
    from unsupervised_growth_gb300 import build
    from unsupervised_growth_gb300.engine import Engine
    build.build()
    e = Engine(precision=64)
    yield e
    e.close()


@pytest.fixture(scope="session")
def engine32():
    from unsupervised_growth_gb300 import build
    from unsupervised_growth_gb300.engine import Engine
    build.build()
    e = Engine(precision=32)
    yield e
    e.close()
