"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the built libmcfd.so; all others
run on a CPU-only host.  The oracle (oracle/liborc.so) is built on demand by
make; libmcfd.so is built on demand by nvcc (cross-compiles without a GPU).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libmcfd.so")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def mcfd_lib():
    from pvcriemannsolvers_gb300 import build, capi
    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def gpu(mcfd_lib):
    if not has_gpu():
        pytest.fail("a CUDA GPU is required for tests marked gpu")
    return mcfd_lib
