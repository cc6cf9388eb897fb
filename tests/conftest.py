import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build_port()
    return oracle


def load_golden(name):
    import numpy as np
    d = dict(np.load(os.path.join(GOLDEN, name)))
    if "w" in d and d["w"].size == 0:
        d["w"] = None
    return d


def canonical_ids(x):
    """Maps every seed index to the lowest index with the same coordinates
    (duplicated seeds are interchangeable as neighbours)."""
    import numpy as np
    _, first, inv = np.unique(x, axis=0, return_index=True, return_inverse=True)
    return first[inv.reshape(-1)].astype(np.uint32)
