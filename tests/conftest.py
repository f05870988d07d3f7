import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def ref():
    """The f32 restatement of the reference step (oracle/lenia_oracle.c)."""
    from oracle.oracle import RefF32
    return RefF32()


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load the engine library; CPU-only tests never launch kernels."""
    from auto_gb300 import native as B
    from auto_gb300 import _lib
    B.build()
    return _lib.load()
