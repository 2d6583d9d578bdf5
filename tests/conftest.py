"""pytest configuration: the `gpu` marker and shared fixtures."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def gepi():
    """The product package with its native library built."""
    from gepicount_gb300 import build

    build.build()
    import gepicount_gb300

    gepicount_gb300.lib()
    return gepicount_gb300


@pytest.fixture(scope="session")
def orc():
    import helpers

    return helpers.oracle()
