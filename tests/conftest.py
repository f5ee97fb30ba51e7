import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def hd():
    """The CUDA engine; GPU tests fail (not skip) when it is missing."""
    import vkhashdag_gb300
    if not os.path.exists(vkhashdag_gb300.library_path):
        from vkhashdag_gb300 import _build
        _build.build()
    vkhashdag_gb300.lib()
    return vkhashdag_gb300
