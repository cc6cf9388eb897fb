"""Laguerre cells for optimal transport and the GPU Newton solver.

Cells with widely spread weights are certified by the power range query
(certification="power_range"); they are compared with the oracle's exact
Laguerre cells, in which every seed clips every cell.  Clipping order
differs (candidates by distance, then the seeds the range query finds), so
volumes agree to rounding (1e-11 relative), neighbour sets exactly.

The solver is checked with the pinned oracle volumes at the weights it returns
(max_i |vol_i - nu_i| / nu_i < 1e-6) and by the oracle's own Newton
solution (weights equal up to the constant the dual leaves free)."""
import numpy as np
import pytest

from conftest import gaussian_mixture

pytestmark = pytest.mark.gpu

VOL_RTOL = 1e-11


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


@pytest.fixture(scope="module")
def ot(oracle_mod):
    from oracle import ot
    return ot


def neighbour_sets(rowptr, nbr, area, n):
    out = []
    for i in range(n):
        a, b = int(rowptr[i]), int(rowptr[i + 1])
        out.append(dict(zip(nbr[a:b].tolist(), area[a:b].tolist())))
    return out


def assert_laguerre_equal(c, r, n):
    vmax = np.max(np.abs(r["vol"]))
    assert np.max(np.abs(c.volume - r["vol"])) <= VOL_RTOL * vmax
    big = r["vol"] > 1e-6 * vmax
    mg_err = np.abs(c.mg - r["mg"]).max(1)
    assert np.max(mg_err[big] / r["vol"][big]) < 1e-9
    A = neighbour_sets(c.rowptr, c.neighbors, c.facet_area, n)
    B = neighbour_sets(r["rowptr"], r["nbr"], r["area"], n)
    amax = max(r["area"].max(), 1e-300)
    for i in range(n):
        # facets of zero area may or may not appear, depending on the order
        a = {j: v for j, v in A[i].items() if v > 1e-12 * amax}
        b = {j: v for j, v in B[i].items() if v > 1e-12 * amax}
        assert a.keys() == b.keys(), i
        for j in a:
            assert abs(a[j] - b[j]) <= 1e-9 * amax


WEIGHT_CASES = {
    # (seed generator, weight generator)
    "uniform_small_w": (lambda r: r.random((1500, 3)), lambda r, n: r.uniform(0, 1e-4, n)),
    "uniform_spread_w": (lambda r: r.random((1500, 3)), lambda r, n: r.uniform(-0.02, 0.02, n)),
    "mixture_spread_w": (lambda r: gaussian_mixture(1500, 8, 0.05, r),
                         lambda r, n: r.uniform(-0.05, 0.05, n)),
}


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", sorted(WEIGHT_CASES))
def test_power_range_cells_vs_oracle(g, ot, case, prec):
    rng = np.random.default_rng(11)
    gx, gw = WEIGHT_CASES[case]
    x = gx(rng)
    w = gw(rng, len(x))
    r = ot.laguerre_cells(x, w)
    c = g.compute_cells(x, w, precision=prec, certification="power_range")
    assert_laguerre_equal(c, r, len(x))
    assert abs(c.volume.sum() - 1.0) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_power_range_cells_vs_reference_fixture(g, prec):
    """At optimal-transport weights, against geogram's own cells (every seed
    a candidate; tests/golden/cells_laguerre_ot_1200.npz)."""
    from conftest import load_golden
    r = load_golden("cells_laguerre_ot_1200.npz")
    c = g.compute_cells(r["x"], r["w"], precision=prec, certification="power_range")
    assert_laguerre_equal(c, r, len(r["x"]))
    assert np.max(np.abs(c.volume * len(r["x"]) - 1.0)) < 1e-8


def test_power_range_equals_security_radius_on_voronoi(g):
    """Zero weights: both certifications give the same cells."""
    x = np.random.default_rng(5).random((3000, 3))
    a = g.compute_cells(x, precision="fp32")
    b = g.compute_cells(x, precision="fp32", certification="power_range")
    assert np.max(np.abs(a.volume - b.volume)) <= VOL_RTOL * a.volume.max()
    A = neighbour_sets(a.rowptr, a.neighbors, a.facet_area, len(x))
    B = neighbour_sets(b.rowptr, b.neighbors, b.facet_area, len(x))
    assert all(p.keys() == q.keys() for p, q in zip(A, B))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_certification_rounds_resume_bit_identical(g, prec, monkeypatch):
    """Cells to which the range query adds candidates continue from their
    polytope of the round before; clipping them again from the box
    (GBV_CERT_RESUME=0) gives the same bits."""
    rng = np.random.default_rng(12)
    x = gaussian_mixture(20000, 8, 0.05, rng)
    w = rng.uniform(-0.01, 0.01, len(x))
    a = g.compute_cells(x, w, precision=prec, certification="power_range")
    monkeypatch.setenv("GBV_CERT_RESUME", "0")
    b = g.compute_cells(x, w, precision=prec, certification="power_range")
    assert a.report["n_more_k"] > 1000  # rounds with many re-clipped cells
    for f in ("volume", "mg", "rowptr", "neighbors", "facet_area", "status"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    monkeypatch.delenv("GBV_CERT_RESUME")
    w1, rep1 = g.ot_solve(x, tol=1e-7)
    monkeypatch.setenv("GBV_CERT_RESUME", "0")
    w0, rep0 = g.ot_solve(x, tol=1e-7)
    assert rep1["converged"] == 1 and rep0["converged"] == 1
    assert np.array_equal(w1, w0)
    assert rep1["newton_iters"] == rep0["newton_iters"]


def test_gradient_and_hessian_vs_oracle(g, ot):
    rng = np.random.default_rng(2)
    x = gaussian_mixture(1200, 6, 0.06, rng)
    w = rng.uniform(-0.02, 0.02, len(x))
    grad, (rp, col, val, diag) = g.ot_gradient_hessian(x, w)
    r = ot.laguerre_cells(x, w)
    n = len(x)
    assert np.max(np.abs(grad - (1.0 / n - r["vol"]))) <= VOL_RTOL * r["vol"].max()
    Hr = ot.hessian(x, r)
    # same operator: compare H d on random vectors and the diagonals
    for _ in range(3):
        d = rng.standard_normal(n)
        y = diag * d
        np.add.at(y, np.repeat(np.arange(n), np.diff(rp.astype(np.int64))), val * d[col])
        yr = ot.spmv(Hr, d)
        assert np.max(np.abs(y - yr)) <= 1e-9 * np.max(np.abs(yr))
    assert np.max(np.abs(diag - Hr[3])) <= 1e-9 * Hr[3].max()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_ot_solve_reaches_mass_tolerance(g, ot, prec):
    rng = np.random.default_rng(0)
    x = gaussian_mixture(3000, 8, 0.05, rng)
    w, rep = g.ot_solve(x, tol=1e-6, precision=prec)
    assert rep["converged"] == 1, rep
    assert rep["mass_error_inf"] < 1e-6
    v = ot.laguerre_cells(x, w)["vol"]
    assert np.max(np.abs(v * len(x) - 1.0)) < 1e-6


def test_ot_solve_matches_oracle_newton(g, ot):
    """The oracle's own Newton solution: the same weights up to a constant."""
    rng = np.random.default_rng(1)
    x = gaussian_mixture(500, 6, 0.05, rng)
    w, rep = g.ot_solve(x, tol=1e-10, precision="fp64")
    assert rep["converged"] == 1, rep
    wr, info = ot.newton(x, tol=1e-10)
    assert info["converged"]
    d = (w - w.mean()) - (wr - wr.mean())
    assert np.max(np.abs(d)) < 1e-7 * (wr.max() - wr.min())


def test_ot_solve_device_matches_host(g):
    import torch
    rng = np.random.default_rng(4)
    x = gaussian_mixture(5000, 5, 0.08, rng)
    nu = rng.uniform(0.5, 1.5, len(x))
    nu /= nu.sum()
    w_h, rep_h = g.ot_solve(x, nu, tol=1e-7)
    xd = torch.tensor(x, device="cuda")
    wd = torch.zeros(len(x), dtype=torch.float64, device="cuda")
    nud = torch.tensor(nu, device="cuda")
    rep_d = g.ot_solve_device(xd, wd, nud, tol=1e-7)
    assert rep_h["converged"] == 1 and rep_d["converged"] == 1
    assert np.array_equal(wd.cpu().numpy(), w_h)
    assert rep_h["newton_iters"] == rep_d["newton_iters"]


def test_warm_start_from_solution_needs_no_step(g):
    rng = np.random.default_rng(6)
    x = gaussian_mixture(2000, 4, 0.07, rng)
    w, rep = g.ot_solve(x, tol=1e-8)
    assert rep["converged"] == 1
    w2, rep2 = g.ot_solve(x, w0=w, tol=1e-6)
    assert rep2["newton_iters"] == 0 and rep2["converged"] == 1
    assert np.array_equal(w2, w)


@pytest.mark.parametrize("nu_kind", ["uniform", "random"])
def test_multilevel_solve(g, ot, nu_kind):
    """optimize_levels: coarse-to-fine; the finest level must reach the
    tolerance, checked with the oracle's volumes."""
    rng = np.random.default_rng(8)
    x = gaussian_mixture(6000, 6, 0.06, rng)
    nu = None
    if nu_kind == "random":
        nu = rng.uniform(0.5, 1.5, len(x))
        nu /= nu.sum()
    w, rep = g.ot_solve_levels(x, nu, ratio=4, min_level=400, tol=1e-6)
    assert rep["levels"] == 2 and rep["converged"] == 1, rep  # 6000 -> 1500 (-> 375 < 400)
    v = ot.laguerre_cells(x, w)["vol"]
    target = np.full(len(x), 1.0 / len(x)) if nu is None else nu
    assert np.max(np.abs(v - target) / target) < 1e-6
