import importlib.util
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libissm103.so")


def load_package():
    """Import the package directory (its name holds a dot) as `issm`."""
    import __graft_entry__

    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as fh:
        data = json.load(fh)
    return {c["name"]: c for c in data["cases"]}


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def issm():
    return load_package()


@pytest.fixture(scope="session")
def cuda(issm):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    issm.native.require()
    return torch.device("cuda:0")
