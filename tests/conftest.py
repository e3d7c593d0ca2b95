import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def gpu():
    """Build the native library (in-tree) and return the package; GPU tests
    fail loudly when CUDA or the library is missing."""
    import torch
    assert torch.cuda.is_available(), "GPU test selected but no CUDA device is visible"
    import __graft_entry__
    __graft_entry__.build()
    import tncontract_gb300 as tn
    torch.cuda.set_device(0)
    return tn
