"""gbv_ot_separable_start: starting weights from the seeds' marginal CDFs.

w = |p|^2 - 2 sum_a Phi_a(p_a), Phi_a' the piecewise-linear empirical CDF
of axis a.  phi = sum_a Phi_a is convex with its gradient inside the box at
every seed, so no cell is empty for distinct seeds (oracle/ot.py,
separable_start, states the argument).  The GPU weights are compared with
the oracle's (equal up to the free constant, to rounding: the prefix sums
run in a different order), the cells at those weights are checked to be all
non-empty on tight clusters, and Newton from them must converge.  The file
runs after the other GPU files."""
import numpy as np
import pytest

from conftest import gaussian_mixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


@pytest.fixture(scope="module")
def ot(oracle_mod):
    from oracle import ot
    return ot


def start(g, x, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))):
    import torch
    return g.ot_separable_start_device(torch.tensor(x, device="cuda"), box=box).cpu().numpy()


@pytest.mark.parametrize("n,sigma,snap", [(1, 0.0, 0), (2, 0.0, 0), (1000, 0.03, 0),
                                          (3001, 0.02, 0), (2000, 0.03, 32)])
def test_matches_oracle(g, ot, n, sigma, snap):
    rng = np.random.default_rng(n)
    x = gaussian_mixture(n, 4, sigma, rng) if sigma else rng.random((n, 3))
    if snap:   # many equal coordinates on every axis
        x = (np.floor(x * snap) + 0.5) / snap
        x[:, 0] += rng.random(n) * 1e-3
    for lo, hi in (((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ((-1.0, 0.0, 2.0), (1.0, 3.0, 5.0))):
        xx = np.asarray(lo) + x * (np.asarray(hi) - np.asarray(lo))
        w = start(g, xx, (lo, hi))
        o = ot.separable_start(xx, lo, hi)
        d = (w - w.mean()) - o
        assert np.max(np.abs(d)) <= 1e-12 * max(1.0, np.max(np.abs(o)))


@pytest.mark.parametrize("sigma", [0.005, 0.02])
def test_no_empty_cell(g, sigma):
    x = gaussian_mixture(20000, 8, sigma, np.random.default_rng(3))
    w = start(g, x)
    c = g.compute_cells(x, w, precision="fp32", certification="power_range")
    assert (c.volume > 0).all()
    assert abs(c.volume.sum() - 1.0) < 1e-10


def test_newton_from_separable_start(g):
    import torch
    x = gaussian_mixture(20000, 8, 0.05, np.random.default_rng(4))
    xd = torch.tensor(x, device="cuda")
    w = g.ot_separable_start_device(xd)
    rep = g.ot_solve_device(xd, w, tol=1e-6)
    assert rep["converged"] and rep["mass_error_inf"] < 1e-6
    c = g.compute_cells(x, w.cpu().numpy(), precision="fp64", certification="power_range")
    assert np.max(np.abs(c.volume * len(x) - 1.0)) < 1e-6
