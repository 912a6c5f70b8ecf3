import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "tight-binding_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def ctx():
    from nrltb import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ex1():
    from nrltb import read_skin
    return read_skin(os.path.join(GOLDEN, "ex1", "SKIN"))


@pytest.fixture(scope="session")
def ex1_gold():
    import json
    with open(os.path.join(GOLDEN, "ex1_golden.json")) as f:
        return json.load(f)
