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


@pytest.mark.parametrize("sigma,snap", [(0.005, 0), (0.02, 0), (0.05, 64)])
def test_separable_start_empties_no_cell(ot, sigma, snap):
    """No empty cell from the separable start, for tight clusters and for seeds
    sharing coordinates (snapped to a 64-grid: many ties on every axis)."""
    rng = np.random.default_rng(11)
    x = gaussian_mixture(500, 8, sigma, rng)
    if snap:
        x = (np.floor(x * snap) + 0.5) / snap
        x[:, 0] += rng.random(len(x)) * 1e-3   # keep the seeds distinct
    w = ot.separable_start(x)
    c = ot.laguerre_cells(x, w)
    assert (c["vol"] > 0).all()
    assert abs(c["vol"].sum() - 1.0) < 1e-12
    # the certificate point grad phi(p_i) = (F_a(p_ia)) lies in cell i
    n = len(x)
    g = np.empty_like(x)
    for a in range(3):
        o = np.argsort(x[:, a], kind="stable")
        g[o, a] = (np.arange(n) + 0.5) / n
    pw = ((g[:, None, :] - x[None, :, :]) ** 2).sum(2) - w[None, :]
    assert (pw.argmin(1) == np.arange(n)).all()


def test_newton_from_separable_start(ot):
    """Same solution as from zero (unique up to a constant), fewer cell passes."""
    rng = np.random.default_rng(0)
    x = gaussian_mixture(400, 8, 0.02, rng)
    w0, i0 = ot.newton(x, tol=1e-8)
    w1, i1 = ot.newton(x, w0=ot.separable_start(x), tol=1e-8)
    assert i0["converged"] and i1["converged"]
    d = (w1 - w1.mean()) - (w0 - w0.mean())
    assert np.max(np.abs(d)) < 1e-6 * np.ptp(w0)
    assert i1["cell_calls"] <= i0["cell_calls"]
