"""The oracle's CPU restatement against the reference's own results.

The golden fixtures were produced by geogram's BalancedKdTree and
VBW::ConvexCell themselves (tests/golden/make_golden.py, oracle/_ref); the
restatement must reproduce them bit for bit on non-degenerate inputs, and
the cell volumes on degenerate ones (a lattice, where equidistant
neighbours are ordered differently: the kd-tree by traversal, the oracle by
index).  When the reference build is present the same is checked live."""
import numpy as np
import pytest

from conftest import canonical_ids, load_golden

EXACT_CASES = ["uniform_1500", "power_1500", "clustered_1500", "shell_901", "shell_1601"]


@pytest.mark.parametrize("name", EXACT_CASES)
def test_port_matches_reference_fixture(oracle_mod, name):
    g = load_golden(f"cells_{name}.npz")
    r = oracle_mod.cells(g["x"], g["w"], nthreads=4)
    for key in ("vol", "mg", "rowptr", "nbr", "area", "status", "n_clip", "k_list"):
        assert np.array_equal(r[key], g[key]), key


def test_port_matches_reference_with_duplicates(oracle_mod):
    """Copies of a seed are equidistant ties: which copy names a facet
    follows the tie order, so neighbours are compared up to duplicates."""
    g = load_golden("cells_duplicates_405.npz")
    r = oracle_mod.cells(g["x"], None, nthreads=4)
    canon = canonical_ids(g["x"])
    for key in ("vol", "mg", "rowptr", "area", "status", "n_clip", "k_list"):
        assert np.array_equal(r[key], g[key]), key
    assert np.array_equal(canon[r["nbr"]], canon[g["nbr"]])


def test_port_matches_reference_on_lattice(oracle_mod):
    g = load_golden("cells_lattice_216.npz")
    r = oracle_mod.cells(g["x"], None, nthreads=4)
    # tie order changes the fan decomposition: equal up to rounding
    assert np.max(np.abs(r["vol"] - g["vol"]) / g["vol"]) < 1e-12
    assert np.max(np.abs(r["mg"] - g["mg"])) < 1e-15
    assert np.array_equal(r["rowptr"], g["rowptr"])
    assert np.max(np.abs(np.sort(r["area"]) - np.sort(g["area"]))) < 1e-15
    assert r["n_exact"] > 0  # the exact predicates were exercised
    assert abs(r["vol"].sum() - 1.0) < 1e-14


@pytest.mark.parametrize("name", ["knn_2000", "knn4_2000"])
def test_port_knn_matches_reference_fixture(oracle_mod, name):
    g = load_golden(f"{name}.npz")
    idx, d2 = oracle_mod.knn(g["x"], 21, nthreads=4)
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(d2, g["d2"])


def test_volume_invariant(oracle_mod):
    """Sum of the cell volumes is the box volume (periodic_delaunay_3d.cpp:4345-4355)."""
    x = np.random.default_rng(5).random((800, 3))
    r = oracle_mod.cells(x, nthreads=4)
    assert abs(r["vol"].sum() - 1.0) < 1e-13
    # adjacency is symmetric
    rows = np.repeat(np.arange(800), np.diff(r["rowptr"]))
    pairs = set(zip(rows.tolist(), r["nbr"].tolist()))
    assert all((j, i) in pairs for i, j in pairs)


def test_det4_exact_sign(oracle_mod):
    # singular (two equal rows) -> 0; identity -> +1; a tiny perturbation
    # of a singular matrix beyond double filters -> its true sign
    a = [1.0, 2.0, 3.0, 4.0]
    b = [0.5, 0.25, 0.125, 1.0]
    c = [3.0, 1.0, 4.0, 1.0]
    assert oracle_mod.det4_sign(a, a, b, c) == 0
    assert oracle_mod.det4_sign([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]) == 1
    d = [x + y for x, y in zip(a, b)]
    eps = 2.0 ** -50  # representable next to 1.5, far below the filter bound
    assert oracle_mod.det4_sign(a, b, c, [d[0] + eps, d[1], d[2], d[3]]) != 0
    assert oracle_mod.det4_sign(a, b, c, d) == 0


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).ref_available()")
def test_port_matches_reference_live(oracle_mod):
    x = np.random.default_rng(11).random((3000, 3))
    w = np.random.default_rng(12).random(3000) * 2e-3
    for ww in (None, w):
        a = oracle_mod.cells(x, ww, nthreads=8, which="ref")
        b = oracle_mod.cells(x, ww, nthreads=8, which="port")
        for key in ("vol", "mg", "rowptr", "nbr", "area", "status", "n_clip", "k_list"):
            assert np.array_equal(a[key], b[key]), key


def test_port_matches_reference_laguerre_fixture(oracle_mod):
    """Laguerre cells with every seed as candidate (the cells of the OT
    solver), at optimal-transport weights: bit for bit against geogram."""
    g = load_golden("cells_laguerre_ot_1200.npz")
    n = len(g["x"])
    r = oracle_mod.cells(g["x"], g["w"], k0=n - 1, check_sr=False, nthreads=4)
    for key in ("vol", "mg", "rowptr", "nbr", "area", "status", "n_clip", "k_list"):
        assert np.array_equal(r[key], g[key]), key


def test_reference_confirms_ot_weights():
    """The fixture's weights come from the OT restatement; the reference's
    own cells at those weights have volume 1/n: the solution satisfies the
    mass condition by geogram's ConvexCell, not only by the oracle's."""
    g = load_golden("cells_laguerre_ot_1200.npz")
    n = len(g["x"])
    assert np.max(np.abs(g["vol"] * n - 1.0)) < 1e-8
    assert abs(g["vol"].sum() - 1.0) < 1e-12


@pytest.mark.parametrize("name,volume", [("cube_300", 1.0), ("lshape_500", 0.75)])
def test_restricted_fixtures_consistent(name, volume):
    """The reference's restricted cells tile their domain; on the cube, where
    every restricted cell is convex and holds its seed, its CVT gradient is
    2 (m p - mg) (RVD.cpp:792-870).  (On the L-shape it is not: the
    reference fans each cell's border from the seed with unsigned volumes.)"""
    from conftest import load_golden
    d = load_golden(f"rvd_{name}.npz")
    assert abs(d["m"].sum() - volume) < 1e-12
    if name == "cube_300":  # convex cells: the exact gradient
        assert np.max(np.abs(d["g"] - 2 * (d["m"][:, None] * d["x"] - d["mg"]))) < 1e-15


@pytest.mark.parametrize("name,src", [("fast_clustered_1500", "clustered_1500"),
                                      ("walk_power_1500", "power_1500"),
                                      ("fastwalk_uniform_1500", "uniform_1500")])
def test_fast_and_walk_variants_pinned(oracle_mod, name, src):
    """The reference's inexact predicates and its walk-based
    clip_by_plane_fast give, on these non-degenerate sets, the exact scan's
    cells bit for bit (fixtures from the reference build); the port in its
    fast mode reproduces them."""
    f, e = load_golden(f"cells_{name}.npz"), load_golden(f"cells_{src}.npz")
    for key in ("vol", "mg", "rowptr", "nbr", "area", "status"):
        assert np.array_equal(f[key], e[key]), key
    r = oracle_mod.cells(f["x"], f["w"], exact=bool(f["exact"]), nthreads=4)
    assert np.array_equal(r["vol"], f["vol"]) and np.array_equal(r["nbr"], f["nbr"])
    assert np.array_equal(r["area"], f["area"])


@pytest.mark.parametrize("name", ["periodic_1000", "periodic_power_1000"])
def test_periodic_fixtures_consistent(name):
    """The reference's periodic cells tile the unit torus, and each facet is
    seen from its other side with the opposite image translation."""
    d = load_golden(f"{name}.npz")
    n = len(d["x"])
    assert abs(d["vol"].sum() - 1.0) < 1e-12
    rp = d["rowptr"].astype(np.int64)
    row = np.repeat(np.arange(n), np.diff(rp))
    sh = d["shift"].astype(np.int64)
    fwd = (row * n + d["nbr"]) * 27 + sh
    back = (d["nbr"].astype(np.int64) * n + row) * 27 + (26 - sh)
    assert np.array_equal(np.sort(fwd), np.sort(back))
