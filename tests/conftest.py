"""Test configuration: the ``gpu`` marker and the in-tree import path.

Tests marked ``gpu`` need a CUDA device and call the library through its
C-ABI; everything else runs on the CPU (the oracle, the host-side analysis,
and that the library loads and exports every declared symbol).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_library():
    from fastode_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("the gpu tests need a CUDA device")
    from fastode_gb300 import build
    build.build()
    return torch
