import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built engine library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def reference_core(oracle):
    core = oracle.ref()
    if core is None:
        pytest.skip("reference core (oracle/_ref) not built on this machine")
    return core


@pytest.fixture(scope="session")
def engine_lib():
    """The CUDA engine (C-ABI library).  GPU tests fail loudly without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gplsaco_gb300 import _lib
    return _lib.load()
