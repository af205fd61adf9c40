"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and call the engine through the C-ABI
(librett.so); everything else runs on the CPU.  The library and the C oracle
are built on first use (incremental).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls the engine's kernels")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    from librett_gb300.build import build
    from oracle.oracle import build_oracle

    build()
    build_oracle()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
