"""Shared fixtures.  Tests marked `gpu` need a GB300 and the built
libcadr_cuda.so; every other test runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(with_ref=True)
    return oracle.load()


@pytest.fixture(scope="session")
def cuda_lib():
    from cadr_gb300 import build
    build.build()
    from cadr_gb300 import lib
    return lib.load()


@pytest.fixture(scope="session")
def ctx(cuda_lib, oracle_lib):
    from cadr_gb300 import lib
    c = lib.Context(0)
    yield c
    c.close()
