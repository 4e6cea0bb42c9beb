import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS, os.path.join(TESTS, "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def small_model_path(tmp_path_factory):
    """The seeded 32-channel, 3-species model of the 64-atom workload (regenerated, ~2 s)."""
    from make_golden import small_model
    return small_model(str(tmp_path_factory.mktemp("models") / "small.json"))


@pytest.fixture(scope="session")
def small_golden():
    import numpy as np
    return dict(np.load(os.path.join(TESTS, "golden", "small_golden.npz")))


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load the engine library; GPU tests only."""
    from symmetrix_gb300.build import build
    build()
    from symmetrix_gb300 import _lib
    return _lib.load()
