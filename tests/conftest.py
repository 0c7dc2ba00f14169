import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs on the GPU box")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as ge
    return ge.load_package()


@pytest.fixture(scope="session")
def lib_path(pkg):
    """The compiled CUDA library (built here if missing; nvcc cross-compiles)."""
    p = pkg.build.lib_path()
    if not p.exists():
        p = pkg.build.build()
    return p


@pytest.fixture(scope="session")
def cuda(pkg, lib_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    pkg.library(path=lib_path)
    return torch


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle
