import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA kernels)")


@pytest.fixture(scope="session")
def gb300_lib():
    """The built C-ABI library (built on first use; no fallback)."""
    from sundials_gb300 import build, load
    if not build.LIB.exists():
        build.build_library()
    return load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import port
    return port.lib()
