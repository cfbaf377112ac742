import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle

    r = oracle.reference()
    if r is None:
        pytest.skip("the reference library is only built where the reference sources are present")
    return r


@pytest.fixture(scope="session")
def ctx():
    from pagmo2_gb300 import _native as N

    c = N.Context(0)
    yield c
    c.close()
