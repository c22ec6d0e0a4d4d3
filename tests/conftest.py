import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native parts once per session (incremental; seconds when up to date)."""
    from annealing_gb300 import _build

    _build.build_all()
    yield


@pytest.fixture(scope="session")
def ctx():
    import annealing_gb300 as sb

    c = sb.Context(0)
    yield c
    c.close()
