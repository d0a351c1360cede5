import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library and the C oracle (idempotent)."""
    from graphalgo_gb300 import build as gbuild
    import oracle
    gbuild.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import graphalgo_gb300 as ga
    c = ga.Context(0)
    yield c
    c.close()
