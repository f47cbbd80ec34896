import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def E():
    """The elfel_gb300 package (host mirror + C-ABI bindings)."""
    return entry.package()


@pytest.fixture(scope="session")
def O():
    """The CPU oracle."""
    return entry.oracle()


@pytest.fixture(scope="session")
def golden():
    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        with open(os.path.join(d, name)) as f:
            return json.load(f)

    return load


@pytest.fixture(scope="session")
def gpu(E):
    """A device context; builds the library if needed."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    E.build()
    return E.default_context(0)
