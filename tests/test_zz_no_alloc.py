"""gbv_knn_noalloc: the allocation-free kNN entry point.

Some callers cannot allocate GPU memory while they run (a strict device
memory budget, their own memory pool, regions where an allocation's implicit
synchronisation is not allowed).  gbv_knn_noalloc keeps all its scratch in a
fixed array inside the library; these tests call it through the C ABI on
device arrays, twice in a row with different point sets (the shared scratch
keeps the previous call's contents, so the second call checks that nothing
stale leaks through), and compare it with the allocating entry points
(gbv_nn_set_points + gbv_nn_get_nearest_neighbors_all), which must agree
exactly: same indices, same squared distances."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 32768


def _noalloc(lib, pts_dev, n, dim, k, stream=None):
    import torch
    idx = torch.empty((n, k), dtype=torch.int32, device=pts_dev.device)
    d2 = torch.empty((n, k), dtype=torch.float64, device=pts_dev.device)
    st = lib.gbv_knn_noalloc(ctypes.c_void_p(pts_dev.data_ptr()), n, dim, pts_dev.shape[1], k,
                             ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(d2.data_ptr()),
                             stream)
    return st, idx, d2


def _allocating(pts, dim, k):
    import geogram_gb300 as g
    nn = g.NearestNeighborSearch(dim)
    nn.set_points(pts)
    return nn.get_nearest_neighbors_by_index(k)


def test_noalloc_matches_allocating_path_twice():
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(123)
    cases = [(rng.random((20000, 3)), 3, 24),
             (np.concatenate([rng.random((5000, 3)), rng.random((5000, 1)) * 0.01], 1), 4, 64)]
    for pts, dim, k in cases:
        dev = torch.from_numpy(pts).cuda()
        st, idx, d2 = _noalloc(lib, dev, len(pts), dim, k)
        assert st == 0, lib.gbv_last_error()
        torch.cuda.synchronize()
        ref_idx, ref_d2 = _allocating(pts, dim, k)
        assert np.array_equal(idx.cpu().numpy().astype(np.uint32), ref_idx)
        assert np.array_equal(d2.cpu().numpy(), ref_d2)


def test_noalloc_rejects_too_many_points():
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    dev = torch.zeros((MAX_POINTS + 1, 3), dtype=torch.float64, device="cuda")
    st, _, _ = _noalloc(lib, dev, MAX_POINTS + 1, 3, 8)
    assert st == 4  # GBV_ERR_CAPACITY
    assert b"32768" in lib.gbv_last_error()
