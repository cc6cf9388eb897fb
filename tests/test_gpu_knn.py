"""GPU NearestNeighborSearch against the reference's kd-tree results."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import geogram_gb300 as g
    return g


@pytest.mark.parametrize("name,dim", [("knn_2000", 3), ("knn4_2000", 4)])
def test_by_index_bit_exact(g, name, dim):
    ref = load_golden(f"{name}.npz")
    nn = g.NearestNeighborSearch(dim)
    nn.set_points(ref["x"])
    idx, d2 = nn.get_nearest_neighbors_by_index(21)
    assert np.array_equal(idx, ref["idx"])
    assert np.array_equal(d2, ref["d2"])


def brute(x, q, k):
    d = (q[:, None, :] - x[None, :, :]) ** 2
    dd = d[..., 0]
    for c in range(1, x.shape[1]):
        dd = dd + d[..., c]
    o = np.lexsort((np.broadcast_to(np.arange(len(x)), dd.shape), dd), axis=1)[:, :k]
    return o, np.take_along_axis(dd, o, 1)


@pytest.mark.parametrize("k", [1, 10, 64, 100])
def test_queries_vs_brute_force(g, k):
    rng = np.random.default_rng(k)
    x = rng.random((3000, 3))
    q = rng.random((500, 3)) * 1.4 - 0.2  # some queries outside the points' box
    nn = g.NearestNeighborSearch(3)
    nn.set_points(x)
    idx, d2 = nn.get_nearest_neighbors(k, q)
    bi, bd = brute(x, q, k)
    assert np.array_equal(idx, bi)
    assert np.array_equal(d2, bd)


def test_clustered_points(g, oracle_mod):
    rng = np.random.default_rng(3)
    c = rng.random((4, 3))
    x = np.clip(c[rng.integers(0, 4, 20000)] + rng.normal(size=(20000, 3)) * 0.01, 0, 1)
    nn = g.NearestNeighborSearch(3)
    nn.set_points(x)
    idx, d2 = nn.get_nearest_neighbors_by_index(30)
    ri, rd = oracle_mod.knn(x, 30, nthreads=8)
    assert np.array_equal(idx, ri)
    assert np.array_equal(d2, rd)


def test_strided_points(g):
    rng = np.random.default_rng(4)
    x = rng.random((1000, 3))
    padded = np.concatenate([x, np.full((1000, 2), 7.0)], axis=1)
    nn = g.NearestNeighborSearch(3)
    nn.set_points(padded.ravel(), stride=5)
    idx, d2 = nn.get_nearest_neighbors_by_index(8)
    nn2 = g.NearestNeighborSearch(3)
    nn2.set_points(x)
    idx2, d22 = nn2.get_nearest_neighbors_by_index(8)
    assert np.array_equal(idx, idx2) and np.array_equal(d2, d22)


def test_errors(g):
    nn = g.NearestNeighborSearch(3)
    with pytest.raises(g.GbvError):
        nn.get_nearest_neighbors(3, np.zeros((1, 3)))  # no points yet
    nn.set_points(np.random.default_rng(0).random((10, 3)))
    with pytest.raises(g.GbvError):
        nn.get_nearest_neighbors(11, np.zeros((1, 3)))  # k > n


@pytest.mark.parametrize("kind", ["uniform", "clustered", "lifted"])
@pytest.mark.parametrize("k", [64, 128])
def test_warp_search_vs_oracle_at_size(g, oracle_mod, kind, k):
    """The warp-synchronous search (all points, sorted slots) on 60k points:
    uniform, tight clusters (leaves far above 32 seeds, many FP32 ties) and
    4-d lifted points, against the oracle's exact lists."""
    rng = np.random.default_rng(k + len(kind))
    n = 60000
    if kind == "clustered":
        c = rng.random((6, 3))
        x = np.clip(c[rng.integers(0, 6, n)] + rng.normal(size=(n, 3)) * 0.003, 0, 1)
    elif kind == "lifted":
        x = np.concatenate([rng.random((n, 3)), np.sqrt(rng.random((n, 1)) * 1e-4)], 1)
    else:
        x = rng.random((n, 3))
    nn = g.NearestNeighborSearch(x.shape[1])
    nn.set_points(x)
    idx, d2 = nn.get_nearest_neighbors_by_index(k)
    ri, rd = oracle_mod.knn(x, k, nthreads=8)
    assert np.array_equal(idx, ri)
    assert np.array_equal(d2, rd)
