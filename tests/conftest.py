import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and libsodagpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads libsodagpu.so; GPU tests use the C ABI through it."""
    from sodabayes_gb300 import build as _b
    _b.build()
    import sodabayes_gb300
    return sodabayes_gb300.library()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O
