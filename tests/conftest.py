import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300")
for p in (PKG_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsgfim.so")


@pytest.fixture(scope="session")
def engine():
    from sgfim.engine import Engine
    eng = Engine(device=0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
