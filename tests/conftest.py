"""Shared test setup: import paths, the `gpu` marker, and builders."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "genesis-2.4_gb300")
ORACLE_DIR = os.path.join(REPO, "oracle")
for p in (REPO, PKG_DIR, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.ensure_built()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_engine():
    import torch  # noqa: F401  (device plumbing only)
    from gbhsolve import engine
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    engine.load()
    return engine
