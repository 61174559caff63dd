"""Shared test setup: the `gpu` marker and import paths.

CPU tests (`-m "not gpu"`) pin the oracle against the reference's own
results and cover host logic; GPU tests (`-m gpu`) are the parity tests of
the CUDA path against the oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build(ref=False) if not os.path.exists(oracle.LIB) else None
    return oracle


@pytest.fixture(scope="session")
def gox():
    import gridoxide_gb300
    from gridoxide_gb300 import build
    build.build()
    return gridoxide_gb300
