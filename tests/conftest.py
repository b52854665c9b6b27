import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblaps_gpu.so")


@pytest.fixture(scope="session")
def lib():
    """The C-ABI library, built in-tree when missing.  No fallback."""
    from laps_gb300 import ffi

    return ffi.load()
