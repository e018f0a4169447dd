import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "gpu-load-balance_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG_DIR, ORACLE_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine():
    import orb_gb300 as E
    E.build()
    E.load()
    return E


@pytest.fixture(scope="session")
def ctx(engine):
    c = engine.Context(0)
    yield c
    c.close()
