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
def predictions():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "predictions_fit03_fit08.npz"))


def channel_weights_for(elements):
    """(channels x elements) weights of the fit08 setup: unweighted, then the weighted_auto pair."""
    import numpy as np
    from mld_gb300 import elements as el
    w2, w3 = el.auto_channel_weights(list(elements))
    return np.stack([np.ones(len(elements)), w2, w3])


@pytest.fixture(scope="session")
def lib():
    from mld_gb300 import build, _lib
    build.build()
    return _lib.load()
