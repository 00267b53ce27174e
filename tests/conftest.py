import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    import json
    here = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(here, "examples.json")) as f:
        ex = json.load(f)
    with open(os.path.join(here, "intersection_kat.json")) as f:
        kat = json.load(f)
    return ex, kat


@pytest.fixture(scope="session")
def counter():
    """A library context on cuda:0.  Fails (does not skip) when the CUDA path cannot load."""
    from katric_gb300 import TriangleCounter
    ctr = TriangleCounter(0)
    yield ctr
    ctr.close()
