import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbims.so")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gblib():
    """Builds (if needed) and loads libgbims.so; GPU tests only."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from modflow6_gb300 import build as b
    b.build()
    from modflow6_gb300 import _lib
    return _lib.load()
