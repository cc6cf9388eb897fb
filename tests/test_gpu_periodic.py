"""Periodic Laguerre cells (gbv_periodic_cells) against the reference's own
PeriodicDelaunay3d + copy_Laguerre_cell_from_Delaunay
(delaunay/periodic_delaunay_3d.cpp:3634-3734) on 1000 seeds in the periodic
unit cube, without and with weights (tests/golden/make_golden.py).  The
reference builds each cell from its Delaunay tetrahedra and the engine clips
it by its ghost-image neighbours in distance order, so the facet sets
(seed, image translation) must be identical and volumes, centroids and
facet areas equal to rounding: 1e-12 relative for volumes and centroids,
1e-10 for facet areas."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


def facets(rowptr, nbr, shift, area, i):
    a, b = int(rowptr[i]), int(rowptr[i + 1])
    keys = nbr[a:b].astype(np.int64) * 27 + shift[a:b]
    o = np.argsort(keys)
    return keys[o], area[a:b][o]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["periodic_1000", "periodic_power_1000"])
def test_periodic_cells_vs_reference(g, name, prec):
    ref = load_golden(f"{name}.npz")
    r = g.periodic_cells(ref["x"], ref["w"], precision=prec)
    assert abs(r["volume"].sum() - 1.0) < 1e-12
    assert np.max(np.abs(r["volume"] - ref["vol"]) / ref["vol"]) < 1e-12
    assert np.max(np.abs(r["mg"] - ref["mg"])) < 1e-12 * ref["vol"].mean()
    for i in range(len(ref["x"])):
        k1, a1 = facets(r["rowptr"], r["neighbors"], r["shift"], r["facet_area"], i)
        k2, a2 = facets(ref["rowptr"], ref["nbr"], ref["shift"], ref["area"], i)
        assert np.array_equal(k1, k2), i
        assert np.max(np.abs(a1 - a2) / a2) < 1e-10, i


def test_periodic_cells_tile_the_torus_at_size(g):
    """100k seeds: volumes sum to the cube's, every facet is seen from both
    sides with opposite translations and the same area."""
    x = np.random.default_rng(11).random((100000, 3))
    r = g.periodic_cells(x, precision="fp32")
    assert abs(r["volume"].sum() - 1.0) < 1e-10
    rp, nb, sh = r["rowptr"].astype(np.int64), r["neighbors"], r["shift"].astype(np.int64)
    row = np.repeat(np.arange(len(x)), np.diff(rp))
    fwd = (row * len(x) + nb) * 27 + sh
    back = (nb.astype(np.int64) * len(x) + row) * 27 + (26 - sh)
    assert np.array_equal(np.sort(fwd), np.sort(back))
