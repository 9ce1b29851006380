"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def native_lib():
    """The compiled library (built here if missing; nvcc cross-compiles)."""
    import synchrowords_gb300 as sw
    from synchrowords_gb300 import build as nb
    nb.build()
    return sw.load_library()


@pytest.fixture(scope="session")
def ctx(native_lib):
    import synchrowords_gb300 as sw
    c = sw.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
