import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def qvectors():
    import numpy as np
    z = np.load(os.path.join(TESTS, "golden", "qvectors3d.npz"))
    return z["n"].astype(np.int32), z["offsets"].astype(np.int32)


@pytest.fixture(scope="session")
def engine_mod():
    """The engine binding; builds the native library if needed (GPU tests only)."""
    from amdat_gb300 import build
    build.build()
    from amdat_gb300 import engine
    return engine


@pytest.fixture()
def eng(engine_mod):
    e = engine_mod.Engine(0)
    yield e
    e.close()
