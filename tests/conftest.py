"""Test configuration.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU (oracle, host logic, library loading).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def built_library():
    from minimc_gb300 import _build

    return _build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build

    return build.load()
