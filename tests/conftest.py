import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The CPU oracle is test infrastructure: build it if it is missing."""
    lib = os.path.join(ROOT, "oracle", "_build", "liboracle32.so")
    if not os.path.exists(lib):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_oracle.sh")], check=True,
                       stdout=subprocess.DEVNULL)
    yield


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
