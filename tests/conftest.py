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


def gaussian_mixture(n, k, sigma, rng, lo=0.2, hi=0.8):
    """n seeds from a k-component isotropic Gaussian mixture (means uniform in
    [lo, hi]^3, standard deviation sigma, or one per component when sigma is
    an array), rejected outside the unit cube."""
    import numpy as np
    mu = rng.uniform(lo, hi, (k, 3))
    sig = np.broadcast_to(np.asarray(sigma, np.float64), (k,))
    out, have = [], 0
    while have < n:
        c = rng.integers(0, k, n)
        p = mu[c] + sig[c, None] * rng.standard_normal((n, 3))
        p = p[((p > 0.0) & (p < 1.0)).all(1)]
        out.append(p)
        have += len(p)
    return np.concatenate(out)[:n]
