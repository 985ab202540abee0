import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine through its C ABI)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle (always) and the engine library (needs nvcc only)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from gpupfem2_gb300 import build as b
    b.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("this test needs a CUDA GPU")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
