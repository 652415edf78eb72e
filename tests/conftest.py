import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.oracle()


@pytest.fixture(scope="session")
def ctx():
    import gasoline_gb300 as g
    c = g.Context(0)
    yield c
    c.close()


@pytest.fixture
def scratch(request):
    """A per-test directory under tests/.scratch for files a test writes."""
    import shutil
    d = os.path.join(ROOT, "tests", ".scratch", request.node.name.replace("/", "_"))
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    yield d
    shutil.rmtree(d, ignore_errors=True)
