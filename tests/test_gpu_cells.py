"""GPU cells through the C ABI against the reference's results.

The fixtures hold geogram's own outputs (BalancedKdTree + VBW::ConvexCell,
tests/golden/make_golden.py).  Both precision modes must reproduce them bit
for bit: neighbour lists, facet areas, volumes and centroids (1e-12
relative would be the bar for volumes and centroids; the engine matches
exactly).  Degenerate inputs (a lattice) are compared on the quantities
that do not depend on how equidistant neighbours are ordered."""
import numpy as np
import pytest

from conftest import canonical_ids, load_golden

pytestmark = pytest.mark.gpu

EXACT_CASES = ["uniform_1500", "power_1500", "clustered_1500", "shell_901", "shell_1601"]
PRECISIONS = ["fp64", "fp32"]


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


def assert_cells_equal(c, ref, nbr=True):
    assert np.array_equal(c.rowptr.astype(np.int64), np.asarray(ref["rowptr"], np.int64))
    if nbr:
        assert np.array_equal(c.neighbors, ref["nbr"])
        assert np.array_equal(c.facet_area, ref["area"])
    assert np.array_equal(c.volume, ref["vol"])
    assert np.array_equal(c.mg, ref["mg"])
    assert np.array_equal(c.status, ref["status"])


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("name", EXACT_CASES)
def test_cells_bit_exact_vs_reference(g, name, prec):
    ref = load_golden(f"cells_{name}.npz")
    c = g.compute_cells(ref["x"], ref["w"], precision=prec)
    assert_cells_equal(c, ref)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_lattice_volumes(g, prec):
    ref = load_golden("cells_lattice_216.npz")
    c = g.compute_cells(ref["x"], precision=prec)
    # equidistant neighbours are ordered differently (kd-tree traversal vs
    # index): the same cells, summed over a different fan decomposition
    assert np.max(np.abs(c.volume - ref["vol"]) / ref["vol"]) < 1e-12
    assert np.array_equal(c.rowptr.astype(np.int64), ref["rowptr"])
    assert c.report["n_exact"] > 0 or prec == "fp32"


@pytest.mark.parametrize("prec", PRECISIONS)
def test_lattice_vs_oracle_bit_exact(g, oracle_mod, prec):
    """On a lattice the oracle orders ties by index like the GPU: identical."""
    gg = (np.arange(7) + 0.5) / 7
    x = np.stack(np.meshgrid(gg, gg, gg, indexing="ij"), -1).reshape(-1, 3)
    r = oracle_mod.cells(x, nthreads=4)
    c = g.compute_cells(x, precision=prec)
    assert_cells_equal(c, r)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("n", [2, 3, 9, 40, 65, 300])
def test_small_n(g, oracle_mod, n, prec):
    x = np.random.default_rng(n).random((n, 3))
    r = oracle_mod.cells(x, nthreads=2)
    c = g.compute_cells(x, precision=prec)
    assert_cells_equal(c, r)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_power_with_empty_cells(g, oracle_mod, prec):
    """Large weights empty some cells; they must come out empty (volume 0)."""
    rng = np.random.default_rng(21)
    x = rng.random((2000, 3))
    w = rng.random(2000) * 0.02
    r = oracle_mod.cells(x, w, nthreads=8)
    c = g.compute_cells(x, w, precision=prec)
    assert (r["vol"] == 0).any()
    assert_cells_equal(c, r)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_without_security_radius(g, oracle_mod, prec):
    """check_sr off: a single pass over the first k0 neighbours (generic_RVD.h:2328)."""
    x = np.random.default_rng(7).random((1000, 3))
    for k0 in (10, 20):
        r = oracle_mod.cells(x, k0=k0, check_sr=False, nthreads=4)
        c = g.compute_cells(x, k0=k0, check_sr=False, precision=prec)
        assert_cells_equal(c, r)


def test_non_unit_box(g):
    """Seeds in [0,2]x[0,1]x[0,3]: the cells tile that box."""
    rng = np.random.default_rng(8)
    x = rng.random((3000, 3)) * np.array([2.0, 1.0, 3.0])
    c = g.compute_cells(x, box=((0, 0, 0), (2, 1, 3)))
    assert abs(c.volume.sum() - 6.0) < 1e-12
    assert (c.status == g.CELL_CERTIFIED).mean() > 0.9


def test_fp32_mode_equals_fp64_mode_at_scale(g):
    rng = np.random.default_rng(9)
    x = rng.random((200_000, 3))
    w = rng.random(200_000) * 1e-4 * 5 ** (2 / 3)
    a = g.compute_cells(x, w, precision="fp64")
    b = g.compute_cells(x, w, precision="fp32")
    assert np.array_equal(a.neighbors, b.neighbors)
    assert np.array_equal(a.volume, b.volume)
    assert np.array_equal(a.mg, b.mg)
    assert b.report["n_recheck_fp64"] < 0.05 * len(x)


def test_size_independent_properties_1m(g):
    """At 1M seeds: total volume 1, symmetric adjacency, matching facet
    areas on both sides, every cell certified or complete."""
    rng = np.random.default_rng(10)
    n = 1_000_000
    x = rng.random((n, 3))
    w = rng.random(n) * 1e-4
    c = g.compute_cells(x, w, precision="fp32")
    assert abs(c.report["volume_sum"] - 1.0) < 1e-12
    assert abs(c.volume.sum() - 1.0) < 1e-11
    assert set(np.unique(c.status)) <= {0, 1}
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(c.rowptr.astype(np.int64)))
    key = rows * n + c.neighbors
    rkey = c.neighbors.astype(np.int64) * n + rows
    o1, o2 = np.argsort(key), np.argsort(rkey)
    assert np.array_equal(key[o1], rkey[o2])
    a1, a2 = c.facet_area[o1], c.facet_area[o2]
    assert np.max(np.abs(a1 - a2) / np.maximum(a1, 1e-300)) < 1e-6


@pytest.mark.parametrize("prec", PRECISIONS)
def test_duplicates_vs_reference(g, oracle_mod, prec):
    """Duplicated seeds: reference fixture up to which copy names a facet,
    and the oracle (same tie order as the GPU) bit for bit."""
    ref = load_golden("cells_duplicates_405.npz")
    c = g.compute_cells(ref["x"], precision=prec)
    canon = canonical_ids(ref["x"])
    assert np.array_equal(c.volume, ref["vol"]) and np.array_equal(c.mg, ref["mg"])
    assert np.array_equal(c.facet_area, ref["area"])
    assert np.array_equal(canon[c.neighbors], canon[ref["nbr"]])
    assert_cells_equal(c, oracle_mod.cells(ref["x"], nthreads=4))


def test_duplicates_status(g):
    ref = load_golden("cells_duplicates_405.npz")
    c = g.compute_cells(ref["x"])
    dup = np.nonzero(c.status == g.CELL_DUPLICATE)[0]
    assert list(dup) == [400, 401, 402, 403, 404]  # the higher-index copies
    # as the reference: the unclipped box (volume 1 up to the fan's rounding)
    assert np.array_equal(c.volume[dup], ref["vol"][dup])
    assert np.allclose(c.volume[dup], 1.0, rtol=0, atol=1e-15)
    # seed 17 has two copies: the reference's list growth stalls at 18
    assert c.status[17] == g.CELL_STALLED and ref["status"][17] == 3


@pytest.mark.parametrize("prec", PRECISIONS)
def test_cells_beyond_fixed_capacity(g, prec):
    """The shell's centre cell (hundreds of facets) and the outer cells with
    more than 64 facets take the unbounded path; results stay bit-exact."""
    ref = load_golden("cells_shell_1601.npz")
    c = g.compute_cells(ref["x"], precision=prec)
    assert c.report["n_huge"] >= 1
    assert np.diff(c.rowptr.astype(np.int64)).max() == np.diff(ref["rowptr"]).max() > 600
    assert_cells_equal(c, ref)


@pytest.mark.parametrize("first_k", [20, 64, 128])
@pytest.mark.parametrize("prec", PRECISIONS)
def test_first_list_length_does_not_change_cells(g, first_k, prec):
    """A first kNN list shorter than most cells need (20: nearly every cell
    grows its list) or long enough for all of them gives the same cells."""
    ref = load_golden("cells_power_1500.npz")
    c = g.compute_cells(ref["x"], ref["w"], precision=prec, first_k=first_k)
    assert_cells_equal(c, ref)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("name", ["fast_clustered_1500", "walk_power_1500",
                                  "fastwalk_uniform_1500"])
def test_fast_predicates_and_walk_vs_reference(g, name, prec):
    """The reference run with use_exact_predicates(false) and/or
    clip_by_plane_fast: the fast-predicate mode (and the default mode for the
    walk) reproduces it bit for bit."""
    ref = load_golden(f"cells_{name}.npz")
    c = g.compute_cells(ref["x"], ref["w"], precision=prec,
                        predicates="exact" if bool(ref["exact"]) else "fast")
    assert_cells_equal(c, ref)


def _far_cutter_case():
    """Seed 0 at (0.3, 0.3, 0.3) with 65,600 seeds packed in [0, 0.1]^3
    behind a guard layer (363 seeds on the faces x, y, z = 0.11) and seed 1
    at (0.9, 0.9, 0.9): seed 0's cell reaches the far corner until seed 1
    cuts it, and seed 1 is the 65,963rd seed of its list."""
    rng = np.random.default_rng(5)
    g1 = np.arange(11) * 0.01 + 0.005
    a, b = np.meshgrid(g1, g1, indexing="ij")
    face = np.stack([np.full(a.size, 0.11), a.ravel(), b.ravel()], 1)
    guards = np.concatenate([face, face[:, [1, 0, 2]], face[:, [1, 2, 0]]])
    x = np.concatenate([[[0.3, 0.3, 0.3], [0.9, 0.9, 0.9]], rng.random((65600, 3)) * 0.1, guards])
    return x


@pytest.fixture(scope="module")
def far_cutter(oracle_mod):
    x = _far_cutter_case()
    pc = oracle_mod.PreparedCells(x, None)
    try:
        r = pc.range(0, 2, 8, max_nbr=4096)
    finally:
        pc.close()
    return x, r


@pytest.mark.parametrize("prec", PRECISIONS)
def test_cutting_plane_beyond_16_bit_list_positions(g, far_cutter, prec):
    """Planes are kept with their 16-bit list position in the fixed-shape
    clipping kernels; a cell cut by a seed further down its list goes to the
    huge-cell kernel and must come out as the oracle's (cells 0 and 1: 364
    and 1 facets, all 65,964 other seeds clipped)."""
    x, r = far_cutter
    c = g.compute_cells(x, precision=prec)
    for k in range(2):
        m = int(r["cnt"][k])
        assert np.array_equal(c.neighbors[c.rowptr[k]:c.rowptr[k + 1]], r["nidx"][k * 4096:k * 4096 + m])
        assert np.array_equal(c.facet_area[c.rowptr[k]:c.rowptr[k + 1]],
                              r["narea"][k * 4096:k * 4096 + m])
        assert c.volume[k] == r["vol"][k]
        assert np.array_equal(c.mg[k], r["mg"][3 * k:3 * k + 3])
    assert 1 in c.neighbors[c.rowptr[0]:c.rowptr[1]]
    assert abs(c.volume.sum() - 1.0) < 1e-9


@pytest.mark.parametrize("case", ["uniform", "power", "clustered"])
def test_fp32_geometry_mode(g, case):
    """GBV_PRECISION_FP32_GEOMETRY: the cells of the FP64 mode (neighbours,
    facets, status identical) with volumes, centroids and facet areas from
    FP32 corners in each seed's frame.  Stated error bars, per cell against
    s_i = max(its FP64 volume, the mean volume 1/n): volume and centroid
    within 1e-4 s_i, facet areas within 1e-3 s_i^(2/3).  The mean volume
    covers tiny Laguerre cells far from their seeds, which carry the FP32
    error of corners at the seed's distance (measured up to 2.4e-3 of their
    own volume, 1.5e-5 of the mean)."""
    rng = np.random.default_rng(31)
    n = 100_000
    if case == "clustered":
        from geogram_gb300.cli import seeds
        x = seeds(n, 8, 0.05, 3)
    else:
        x = rng.random((n, 3))
    w = rng.random(n) * n ** (-2.0 / 3.0) if case == "power" else None
    a = g.compute_cells(x, w, precision="fp64")
    b = g.compute_cells(x, w, precision="fp32_geometry")
    assert np.array_equal(a.status, b.status)
    assert np.array_equal(a.rowptr, b.rowptr)
    assert np.array_equal(a.neighbors, b.neighbors)
    s_i = np.maximum(a.volume, 1.0 / n)
    cell = np.repeat(np.arange(n), np.diff(a.rowptr.astype(np.int64)))
    ev = np.max(np.abs(b.volume - a.volume) / s_i)
    em = np.max(np.abs(b.mg - a.mg).max(axis=1) / s_i)
    ea = np.max(np.abs(b.facet_area - a.facet_area) / s_i[cell] ** (2.0 / 3.0))
    print(f"\n{case}: max errors / s_i: volume {ev:.2e}, mg {em:.2e}; "
          f"facet area / s_i^(2/3) {ea:.2e}")
    assert ev < 1e-4 and em < 1e-4 and ea < 1e-3
    assert abs(b.volume.sum() - 1.0) < 1e-6  # FP32 per cell: measured 4e-8 in all
