import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libddgi.so")


@pytest.fixture(scope="session")
def ctx():
    from anerend_gb300 import ddgi

    c = ddgi.Context(0)
    yield c
    c.close()
