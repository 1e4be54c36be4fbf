import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def umtlib():
    """The CUDA library, built in-tree; GPU tests fail loudly without it."""
    from umt_gb300 import build, capi
    build.build()
    return capi.Library()
