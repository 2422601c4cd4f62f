import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libmsgpu.so")


@pytest.fixture(scope="session")
def ref_tests():
    with open(os.path.join(GOLDEN, "reference_tests.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ref_runs():
    with open(os.path.join(GOLDEN, "reference_runs.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ms():
    """The product package with the device initialised (GPU tests only)."""
    import msmodel_gb300 as m
    m.init(0)
    return m
