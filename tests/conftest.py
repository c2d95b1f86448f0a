"""pytest configuration: the ``gpu`` marker and shared fixtures.

Tests marked ``gpu`` need a CUDA device (the libraries are built for GB300, sm_103a); all other
tests run on a CPU-only machine.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_required():
    if not cuda_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="session")
def built_libraries():
    from bullseye_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def oracle_built():
    from oracle.harness import build_oracle
    build_oracle()
    return True
