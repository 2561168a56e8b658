"""Shared pytest configuration.

``-m gpu`` tests need a CUDA device and the built libzgl.so; everything else
runs on the CPU (oracle, host-side logic, C-ABI symbol checks).
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled libzgl.so")


@pytest.fixture(scope="session")
def zgl_lib():
    """The compiled product library (built on demand)."""
    from zillumgl_gb300 import build as zbuild

    zbuild.build()
    import zillumgl_gb300

    return zillumgl_gb300.lib()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
