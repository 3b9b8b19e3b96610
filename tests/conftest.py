"""Shared pytest setup.

Tests marked ``gpu`` need a CUDA device and call the native library through
its C ABI; everything else runs on a CPU-only machine.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("CUDA not available")
    from page_rank_gb300 import native

    native.lib()  # the GPU tests must run the native library, never a fallback
    return torch.device("cuda")
