"""Test configuration: paths, the gpu marker, and builds of the libraries."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "fedem-solvers_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def _gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_lib():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from oracle import oracle

    return oracle.load()


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA solver core; built here if missing (nvcc cross-compiles)."""
    from fedem_gb300.buildlib import build

    build()
    import fedem_gb300

    return fedem_gb300.load_library()


@pytest.fixture(scope="session")
def gpu(gpu_lib):
    if not _gpu_available():
        pytest.fail("a -m gpu test ran without a CUDA device")
    return gpu_lib
