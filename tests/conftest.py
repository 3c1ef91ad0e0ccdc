import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (a GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """libog.so and the oracle are built once per session (no-op when current)."""
    import __graft_entry__

    __graft_entry__.build()


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


def golden_names(z, key):
    return sorted({k.split("/")[0] for k in z.files if k.endswith("/" + key)})
