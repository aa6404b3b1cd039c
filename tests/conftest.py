import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmld_gpu.so")


@pytest.fixture(scope="session")
def fit17():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "fit17_bso4.npz"))


@pytest.fixture(scope="session")
def fit19():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "fit19_bso4_3ch.npz"))


@pytest.fixture(scope="session")
def lib():
    from mld_gb300 import build, _lib
    build.build()
    return _lib.load()
