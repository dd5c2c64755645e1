import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built CUDA library")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Builds the host library and the oracle once per session (the CUDA library only when a
    GPU is present; on CPU-only machines the GPU tests are skipped)."""
    from plens_gb300 import build
    build.build_host()
    from oracle import pyoracle
    pyoracle.build()
    if _has_gpu():
        build.build_gpu()
    yield
