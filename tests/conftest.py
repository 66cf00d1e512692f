import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def genie():
    """The CUDA library, built for sm_103a and loaded (GPU tests only)."""
    from genie_gb300 import build
    build.build()
    import genie_gb300 as g
    g._check(g.lib().genie_init(0))
    return g


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
