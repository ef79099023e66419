import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests proper")


@pytest.fixture(scope="session")
def ctx():
    from mestrado_gb300 import Context
    c = Context(10, 2)
    yield c
    c.close()
