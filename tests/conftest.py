import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in-tree if missing (nvcc cross-compiles here)."""
    from shadowvm_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def engine_factory(built_lib):
    from shadowvm_gb300 import Engine
    engines = []

    def make(**kw):
        e = Engine(**kw)
        engines.append(e)
        return e

    yield make
    for e in engines:
        e.close()
