import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_golden(L: int) -> dict:
    with np.load(os.path.join(GOLDEN, f"golden_L{L}.npz")) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope="session")
def oracle_built():
    import oracle
    oracle.build()  # the reference part only where its sources exist
    return oracle


@pytest.fixture(scope="session")
def product_built():
    from dynamite_gb300 import build
    build.build()
    import dynamite_gb300
    return dynamite_gb300
