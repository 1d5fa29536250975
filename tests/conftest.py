import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: large problem sizes")


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch  # noqa: F401  (only used to probe the device)
        return torch.cuda.is_available()
    except Exception:
        return False
