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


def _context_with(engine, cta_min_cells):
    old = os.environ.get("ORB_CTA_MIN_CELLS")
    os.environ["ORB_CTA_MIN_CELLS"] = str(cta_min_cells)
    try:
        return engine.Context(0)
    finally:
        if old is None:
            del os.environ["ORB_CTA_MIN_CELLS"]
        else:
            os.environ["ORB_CTA_MIN_CELLS"] = old


@pytest.fixture(scope="session", params=["multi_cta", "cta_per_cell"])
def any_ctx(request, engine):
    """A context forced onto one bisection path for every level: the multi-CTA histogram
    passes, or one CTA per cell."""
    c = _context_with(engine, 1 << 30 if request.param == "multi_cta" else 1)
    yield c
    c.close()
