import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the GB300); the parity tests proper")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """The oracle's restatement and the product library, built in-tree if a previous build() did not."""
    import oracle
    from lizard_gb300 import build
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    build.build()
    yield


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
