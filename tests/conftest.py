import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def vrc_lib():
    from voreen_gb300 import build
    build.build()
    import voreen_gb300
    return voreen_gb300.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(vrc_lib):
    import voreen_gb300 as v
    c = v.Context(0)
    yield c
    c.close()
