import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: full-size workloads")


def _build_all():
    from compute_rasterizer_gb300 import build as b
    from oracle import oracle as o
    b.build()
    o.build()


@pytest.fixture(scope="session", autouse=True)
def built():
    _build_all()
    yield


@pytest.fixture(scope="session")
def ctx(built):
    import compute_rasterizer_gb300 as cr
    c = cr.Context(0)
    yield c
    c.close()
