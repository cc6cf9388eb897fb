"""gbv_knn_noalloc: the allocation-free kNN entry point.

Some callers cannot allocate GPU memory while they run (a strict device
memory budget, their own memory pool, regions where an allocation's implicit
synchronisation is not allowed).  gbv_knn_noalloc keeps all its scratch in a
fixed array inside the library; these tests call it through the C ABI on
device arrays and compare it with the allocating entry points
(gbv_nn_set_points + gbv_nn_get_nearest_neighbors_all), which must agree
exactly: same indices, same squared distances.  Calls come in pairs with
different point sets, because the shared scratch keeps the previous call's
contents and nothing stale may leak through; the sizes reach the scratch's
limits (the largest point count at k = 64, then a coarser grid).  A warm
call must leave the device's free memory unchanged, and the array's address
must still be right after cudaDeviceReset."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
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


def _check_against_allocating(lib, cases):
    import torch
    for pts, dim, k in cases:
        dev = torch.from_numpy(pts).cuda()
        st, idx, d2 = _noalloc(lib, dev, len(pts), dim, k)
        assert st == 0, lib.gbv_last_error()
        torch.cuda.synchronize()
        ref_idx, ref_d2 = _allocating(pts, dim, k)
        assert np.array_equal(idx.cpu().numpy().astype(np.uint32), ref_idx)
        assert np.array_equal(d2.cpu().numpy(), ref_d2)


def test_noalloc_matches_allocating_path_twice():
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(123)
    _check_against_allocating(lib, [
        (rng.random((20000, 3)), 3, 24),
        (np.concatenate([rng.random((5000, 3)), rng.random((5000, 1)) * 0.01], 1), 4, 64)])


def test_noalloc_at_the_limits_then_a_coarser_grid():
    from geogram_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(7)
    # the largest point count (grid level 5) at the largest k, then about
    # 500 points (grid level 3) on the same scratch
    _check_against_allocating(lib, [(rng.random((MAX_POINTS, 3)), 3, 64),
                                    (rng.random((500, 3)), 3, 20)])


def test_noalloc_allocates_nothing():
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(11)
    pts = torch.from_numpy(rng.random((8000, 3))).cuda()
    idx = torch.empty((8000, 32), dtype=torch.int32, device="cuda")
    d2 = torch.empty((8000, 32), dtype=torch.float64, device="cuda")
    args = (ctypes.c_void_p(pts.data_ptr()), 8000, 3, 3, 32, ctypes.c_void_p(idx.data_ptr()),
            ctypes.c_void_p(d2.data_ptr()), None)
    assert lib.gbv_knn_noalloc(*args) == 0, lib.gbv_last_error()  # loads the array
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert lib.gbv_knn_noalloc(*args) == 0, lib.gbv_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_too_many_points():
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    dev = torch.zeros((MAX_POINTS + 1, 3), dtype=torch.float64, device="cuda")
    st, _, _ = _noalloc(lib, dev, MAX_POINTS + 1, 3, 8)
    assert st == 4  # GBV_ERR_CAPACITY
    assert b"32768" in lib.gbv_last_error()


def test_noalloc_rejects_host_arrays():
    """Host memory is refused before anything is launched."""
    import torch

    from geogram_gb300 import _lib
    lib = _lib.load()
    pts = np.random.default_rng(3).random((100, 3))
    idx = torch.empty((100, 8), dtype=torch.int32, device="cuda")
    st = lib.gbv_knn_noalloc(ctypes.c_void_p(pts.ctypes.data), 100, 3, 3, 8,
                             ctypes.c_void_p(idx.data_ptr()), None, None)
    assert st == 1  # GBV_ERR_INVALID_ARGUMENT
    assert b"device memory" in lib.gbv_last_error()


_RESET_CHILD = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from geogram_gb300 import _lib
    from oracle import oracle
    lib = _lib.load()
    rt = ctypes.CDLL("libcudart.so.13")  # the runtime libgbv.so is linked with
    V, S = ctypes.c_void_p, ctypes.c_size_t
    n, k = 3000, 16
    pts = np.random.default_rng(5).random((n, 3))

    def run():
        bufs = [V(), V(), V()]
        for b, nb in zip(bufs, (pts.nbytes, n * k * 4, n * k * 8)):
            assert rt.cudaMalloc(ctypes.byref(b), S(nb)) == 0
        assert rt.cudaMemcpy(bufs[0], V(pts.ctypes.data), S(pts.nbytes), 1) == 0
        st = lib.gbv_knn_noalloc(bufs[0], n, 3, 3, k, bufs[1], bufs[2], None)
        assert st == 0, lib.gbv_last_error()
        assert rt.cudaDeviceSynchronize() == 0
        idx = np.empty((n, k), np.uint32)
        d2 = np.empty((n, k))
        assert rt.cudaMemcpy(V(idx.ctypes.data), bufs[1], S(idx.nbytes), 2) == 0
        assert rt.cudaMemcpy(V(d2.ctypes.data), bufs[2], S(d2.nbytes), 2) == 0
        for b in bufs:
            assert rt.cudaFree(b) == 0
        return idx, d2

    a = run()
    assert rt.cudaDeviceReset() == 0  # ends this process's context only
    b = run()
    ref_idx, ref_d2 = oracle.knn(pts, k, nthreads=4)
    for got in (a, b):
        assert np.array_equal(got[0], ref_idx) and np.array_equal(got[1], ref_d2)
    print("reset ok")
""")


def test_noalloc_after_device_reset():
    """A fresh context (here after cudaDeviceReset, in a child process that
    owns nothing else on the GPU) holds the array at a new address; the call
    must use that one."""
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, ROOT], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reset ok" in r.stdout
