import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def golden_pools():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "bound_pools.npz"))


@pytest.fixture(scope="session")
def golden_explore():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "explore.json")) as f:
        return json.load(f)["runs"]
