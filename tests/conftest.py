import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "heyoka.py_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhyk.so")


@pytest.fixture(scope="session")
def libhyk():
    """libhyk.so, built in-tree if missing or stale."""
    from hyk import _build, _lib

    _build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def pins():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "notebook_pins.json")) as f:
        return json.load(f)
