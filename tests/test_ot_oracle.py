"""The CPU optimal-transport restatement (oracle/ot.py), checked without a GPU.

The reference's solver is absent from its checkout, so OT parity is
unpinned; these tests pin what can be pinned: the Hessian against finite
differences of the cell volumes (which are pinned to the reference's
ConvexCell), the known answer of a lattice, and convergence of the plain
Newton solver to the mass tolerance of the OT workload (1e-6)."""
import numpy as np
import pytest

from conftest import gaussian_mixture


@pytest.fixture(scope="module")
def ot(oracle_mod):
    from oracle import ot
    return ot


def test_lattice_is_optimal(ot):
    g = (np.arange(6) + 0.5) / 6
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    c = ot.laguerre_cells(x, np.zeros(len(x)))
    assert np.max(np.abs(c["vol"] - 1.0 / 216)) < 1e-15
    w, info = ot.newton(x)
    assert info["iters"] == 0 and info["converged"]


def test_hessian_is_the_volume_jacobian(ot):
    rng = np.random.default_rng(3)
    x = gaussian_mixture(300, 6, 0.06, rng)
    w = rng.uniform(-0.01, 0.01, len(x))
    c = ot.laguerre_cells(x, w)
    H = ot.hessian(x, c)
    rp, col, val, diag = H
    # a symmetric Laplacian: zero row sums, non-positive off-diagonal
    row = np.repeat(np.arange(len(x)), np.diff(rp))
    s = diag.copy()
    np.add.at(s, row, val)
    assert np.max(np.abs(s)) < 1e-12 * diag.max()
    assert (val <= 0).all()
    key = dict(zip(zip(row.tolist(), col.tolist()), val.tolist()))
    assert all(key.get((j, i), 0.0) == v for (i, j), v in key.items())
    d = rng.standard_normal(len(x))
    h = 1e-7
    fd = (ot.laguerre_cells(x, w + h * d)["vol"] - ot.laguerre_cells(x, w - h * d)["vol"]) / (2 * h)
    an = ot.spmv(H, d)
    assert np.max(np.abs(fd - an)) < 1e-6 * np.max(np.abs(an))


def test_newton_converges_on_a_mixture(ot):
    rng = np.random.default_rng(0)
    x = gaussian_mixture(400, 8, 0.05, rng)
    w, info = ot.newton(x, tol=1e-6)
    assert info["converged"] and info["mass_error_inf"] < 1e-6
    v = ot.laguerre_cells(x, w)["vol"]
    assert np.max(np.abs(v * len(x) - 1.0)) < 1e-6
    assert abs(v.sum() - 1.0) < 1e-12
