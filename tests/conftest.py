import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libdimgpu.so")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def torch_cuda():
    """torch with a CUDA device; GPU tests must not silently pass without one."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected but no CUDA device is visible")
    return torch


@pytest.fixture(scope="session")
def native():
    """libdimgpu.so, built in-tree if needed.  Fails loudly when it cannot be built or loaded."""
    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300 import _native as N

    return N.lib()


@pytest.fixture(scope="session")
def native_test():
    """libdimgpu_test.so: the library built with test hooks and 20 ms bounded device waits (only for the
    tests that make a wait run out)."""
    from diploma_research_gb300 import build as B

    B.build(variant="test")
    from diploma_research_gb300 import _native as N

    return N.test_lib()
