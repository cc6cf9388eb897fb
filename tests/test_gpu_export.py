"""Cell polytopes through the C ABI (gbv_cells_mesh) against the reference's
own ConvexCell::save output (voronoi/convex_cell.cpp:282-352): the fixtures
hold the text geogram writes for ten cells of the uniform and weighted
1500-seed sets, plain and shrunk (tests/golden/make_golden.py).  The same
text must come out, character for character, in both precision modes."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("src", ["uniform_1500", "power_1500"])
def test_obj_text_equals_reference(g, src, prec):
    ref = load_golden(f"cells_{src}.npz")
    obj = np.load(os.path.join(GOLDEN, f"obj_{src}.npz"))
    c = g.compute_cells(ref["x"], ref["w"], precision=prec)
    which = obj["which"]
    assert g.cells_mesh(which).obj_text() == str(obj["obj"])
    four = which[:4]
    shrunk = g.cells_mesh(four).obj_text(shrink=0.2, barycenters=c.barycenter()[four])
    assert shrunk == str(obj["obj_shrink"])


def test_every_cell_polytope_is_consistent(g):
    """All cells of a weighted set: each polygon's seed set equals the cell's
    facet neighbours, every corner is in exactly three polygons, and the
    polytope is a sphere (V - E + F = 2)."""
    ref = load_golden("cells_power_1500.npz")
    c = g.compute_cells(ref["x"], ref["w"], precision="fp32")
    m = g.cells_mesh()
    assert len(m.cells) == len(ref["x"])
    for k in range(len(m.cells)):
        f0, f1 = int(m.cell_face_ptr[k]), int(m.cell_face_ptr[k + 1])
        v0, v1 = int(m.cell_vertex_ptr[k]), int(m.cell_vertex_ptr[k + 1])
        seeds = m.face_seed[f0:f1]
        nb, _ = c.neighbors_of(k)
        assert sorted(seeds[seeds != 0xFFFFFFFF].tolist()) == sorted(nb.tolist())
        ids = m.face_vertices[m.face_ptr[f0]:m.face_ptr[f1]]
        assert np.array_equal(np.bincount(ids, minlength=v1 - v0), np.full(v1 - v0, 3))
        nv, nf = v1 - v0, f1 - f0
        if nv:
            assert nv - 3 * nv // 2 + nf == 2


def test_mesh_needs_cells(g):
    ctx = g.Context(0)
    with pytest.raises(g.GbvError):
        g.cells_mesh([0], ctx=ctx)
    ctx.close()
