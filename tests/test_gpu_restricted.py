"""Cells restricted to tetrahedral meshes (gbv_restricted_cells) against the
reference's own volumetric RestrictedVoronoiDiagram: the fixtures hold the
masses, first moments, CVT energy and gradient that geogram's Delaunay +
RVD compute (voronoi/RVD.cpp:429-530, :792-910) on the unit cube as six
tetrahedra and on an L-shaped non-convex domain of 288 tetrahedra
(tests/golden/make_golden.py).  The decomposition into pieces differs from
the reference's, so the bar is rounding: 1e-12 relative to the mean cell
mass for m, mg and g, 1e-12 relative for the energy."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["cube_300", "lshape_500"])
def test_restricted_cells_vs_reference(g, name, prec):
    ref = load_golden(f"rvd_{name}.npz")
    r = g.restricted_cells(ref["mesh_xyz"], ref["tets"], ref["x"], precision=prec)
    scale = ref["m"].mean()
    assert np.max(np.abs(r["m"] - ref["m"])) <= 1e-12 * scale
    assert np.max(np.abs(r["mg"] - ref["mg"])) <= 1e-12 * scale
    assert np.max(np.abs(r["g"] - ref["g"])) <= 1e-12 * scale
    assert abs(r["f"] - float(ref["f"])) <= 1e-12 * float(ref["f"])
    assert abs(r["m"].sum() - ref["m"].sum()) <= 1e-13


def test_restricted_cells_in_the_whole_box_are_the_cells(g):
    """On the cube as six tetrahedra, the restricted cells are the cells."""
    ref = load_golden("rvd_cube_300.npz")
    r = g.restricted_cells(ref["mesh_xyz"], ref["tets"], ref["x"])
    c = g.compute_cells(ref["x"])
    assert np.max(np.abs(r["m"] - c.volume) / c.volume) < 1e-12


@pytest.mark.parametrize("name", ["cube_300", "lshape_500"])
def test_cvt_newton_vs_reference(g, name):
    """CVT::Newton_iterations (HLBFGS on the restricted cells' energy and
    gradient, voronoi/CVT.cpp:272-307) against the reference's own run:
    Newton_iterations(1) and (10), the GPU energy and gradient at every
    step; the seeds agree within 1e-9 (the energy and gradient agree to
    1e-12 at each step, the line searches take the same branches)."""
    ref = load_golden(f"cvt_newton_{name}.npz")
    for it in (1, 10):
        x, energy = g.cvt_newton(ref["mesh_xyz"], ref["tets"], ref["x"], it)
        assert len(energy) == it + 2
        assert np.all(np.diff(energy) < 0)
        assert np.max(np.abs(x - ref[f"x{it}"])) < 1e-9
        assert abs(energy[-1] - float(ref[f"f{it}"])) <= 1e-10 * float(ref[f"f{it}"])
