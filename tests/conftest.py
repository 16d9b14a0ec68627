"""Test configuration: the `gpu` marker and the in-tree build.

CPU tests (`-m "not gpu"`) run the oracle against the reference's golden
vectors, the host-side library logic and the C ABI's exports. GPU tests call
the CUDA path through the C ABI and compare it with the oracle.
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from ray_tracing_gb300 import build
    build.build_all()
    yield


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover - torch missing
        return False


@pytest.fixture(scope="session")
def gpu_renderer_factory():
    if not cuda_available():
        pytest.fail("GPU test on a machine without a CUDA device")
    from ray_tracing_gb300.renderer import Renderer

    def make(**kw):
        return Renderer(**kw)
    return make
