import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def zlib():
    """The built native library (built in-tree if needed)."""
    from zisafvm_gb300 import _build
    _build.build()
    import zisafvm_gb300 as z
    z.load_library()
    return z


@pytest.fixture(scope="session")
def olib():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle
