import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def gsls():
    """The product library, built in-tree; GPU tests fail loudly without it."""
    from svfsi_gb300 import _lib, build
    build.build()
    L = _lib.load()
    _lib.check(L.gsls_init(int(os.environ.get("GSLS_DEVICE", "0"))), "gsls_init")
    return L


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.load()
    oracle.set_threads(1)
    return oracle
