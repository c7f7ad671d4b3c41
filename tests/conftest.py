import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "reference: needs the reference built headless under oracle/_ref")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import portbind
    portbind.build()
    return portbind.lib()
