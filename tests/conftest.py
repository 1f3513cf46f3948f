import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 host)")


@pytest.fixture(scope="session")
def oracle():
    import model

    model.lib(64)
    model.lib(32)
    return model


@pytest.fixture(scope="session")
def tomo():
    import tomography_gb300

    tomography_gb300.library()
    return tomography_gb300
