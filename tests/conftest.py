import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size cases")


@pytest.fixture(scope="session")
def stencil_lib():
    """Builds (if stale) and loads the in-tree libstencil_gb300.so."""
    from thesis_gb300 import build, lib
    build.build()
    return lib.load()


@pytest.fixture(scope="session")
def cuda(stencil_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    major, minor = torch.cuda.get_device_capability()
    assert (major, minor) == (10, 3), "built for sm_103a, found sm_%d%d" % (major, minor)
    return torch.device("cuda:0")
