"""Oracle bindings -- TEST INFRASTRUCTURE ONLY.

ctypes access to
  - oracle/libgbv_oracle.so: the CPU restatement of the reference's path
    (oracle/gbv_oracle.c), which runs anywhere gcc does;
  - oracle/_ref/libgbv_ref.so: geogram's own BalancedKdTree and
    VBW::ConvexCell compiled from the reference sources (built only where
    the reference checkout is present).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, to check results.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "libgbv_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libgbv_ref.so")
# the reference checkout: GEOGRAM_SRC in the environment, else the usual
# read-only mount
REF_SRC = os.environ.get("GEOGRAM_SRC", "/root/reference")

_port = None
_ref = None


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return PORT_LIB


def build_ref(jobs: int = 8) -> str | None:
    """Compiles the reference's sources into oracle/_ref (needs the checkout)."""
    if not os.path.isdir(os.path.join(REF_SRC, "src", "lib", "geogram")):
        return None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"-j{jobs}",
                    f"REF={REF_SRC}"], check=True)
    return REF_LIB


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = ctypes.CDLL(PORT_LIB)
        P = ctypes.c_void_p
        U = ctypes.c_uint32
        lib.orc_knn.argtypes = [P, U, U, U, P, P, ctypes.c_int]
        lib.orc_cells.argtypes = [P, P, U, U, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P,
                                  P, P, U, P, P, P, P]
        lib.orc_det4_sign.argtypes = [P, P, P, P]
        lib.orc_cells_range.argtypes = [P, P, U, U, U, U, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, P, P, P, P, P, U, P, P, P, P]
        lib.orc_cells_prepare.argtypes = [P, P, U]
        lib.orc_cells_prepare.restype = ctypes.c_void_p
        lib.orc_cells_release.argtypes = [P]
        lib.orc_cells_release.restype = None
        lib.orc_cells_prepared_range.argtypes = [P, U, U, U, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, P, P, P, P, P, U, P, P, P, P]
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref/libgbv_ref.so is not built")
        lib = ctypes.CDLL(REF_LIB)
        P = ctypes.c_void_p
        U = ctypes.c_uint32
        lib.ref_init.argtypes = []
        lib.ref_knn.argtypes = [P, U, U, U, P, P, ctypes.c_int]
        lib.ref_cells.argtypes = [P, P, U, U, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P,
                                  P, U, P, P, P]
        lib.ref_cells_save.argtypes = [P, P, U, U, ctypes.c_int, P, U, ctypes.c_double, P,
                                       ctypes.c_size_t]
        lib.ref_cells_save.restype = ctypes.c_long
        lib.ref_rvd_volume.argtypes = [P, U, P, U, P, U, P, P, P, P]
        lib.ref_cvt_newton.argtypes = [P, U, P, U, P, U, U, U, P]
        lib.ref_set_walk.argtypes = [ctypes.c_int]
        lib.ref_periodic_cells.argtypes = [P, P, U, ctypes.c_double, P, P, P, P, P, P, U]
        lib.ref_init()
        _ref = lib
    return _ref


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def knn(pts: np.ndarray, k: int, nthreads: int = 1, which: str = "port"):
    """k nearest (self included) of every point, ascending (d2, index)."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, dim = pts.shape
    idx = np.empty((n, k), np.uint32)
    d2 = np.empty((n, k))
    lib = port() if which == "port" else ref()
    fn = lib.orc_knn if which == "port" else lib.ref_knn
    r = fn(_p(pts), dim, n, k, _p(idx), _p(d2), nthreads)
    if r != 0:
        raise RuntimeError("knn failed")
    return idx, d2


def cells(xyz: np.ndarray, w: np.ndarray | None = None, k0: int = 20, check_sr: bool = True,
          exact: bool = True, nthreads: int = 1, which: str = "port", max_nbr: int = 96,
          walk: bool = False) -> dict:
    """Certified cells in the unit box; dict of per-seed arrays plus CSR.
    exact=False: the reference's inexact predicates; walk=True (reference
    build only): clipped by ConvexCell::clip_by_plane_fast."""
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    out = dict(vol=np.zeros(n), mg=np.zeros((n, 3)), cnt=np.zeros(n, np.uint32),
               nidx=np.zeros((n, max_nbr), np.uint32), narea=np.zeros((n, max_nbr)),
               k_list=np.zeros(n, np.uint32), n_clip=np.zeros(n, np.uint32),
               status=np.zeros(n, np.int32))
    args = [_p(x), _p(wa), n, k0, int(check_sr), int(exact), nthreads, _p(out["vol"]),
            _p(out["mg"]), _p(out["cnt"]), _p(out["nidx"]), _p(out["narea"]), max_nbr,
            _p(out["k_list"]), _p(out["n_clip"]), _p(out["status"])]
    if which == "port":
        ne = ctypes.c_long(0)
        r = port().orc_cells(*args, ctypes.byref(ne))
        out["n_exact"] = ne.value
    else:
        ref().ref_set_walk(1 if walk else 0)
        r = ref().ref_cells(*args)
        ref().ref_set_walk(0)
    if r != 0:
        raise RuntimeError("cells failed")
    cnt = out["cnt"].astype(np.int64)
    if (out["status"] == 4).any():
        # a cell with more facets than max_nbr: again with room for all
        return cells(x, wa, k0, check_sr, exact, nthreads, which, int(cnt.max()) + 1, walk)
    rowptr = np.zeros(n + 1, np.int64)
    rowptr[1:] = np.cumsum(cnt)
    mask = np.arange(max_nbr)[None, :] < cnt[:, None]
    out["rowptr"] = rowptr
    out["nbr"] = out["nidx"][mask]
    out["area"] = out["narea"][mask]
    del out["nidx"], out["narea"]
    return out


class PreparedCells:
    """The CPU restatement's seed set with its grid built once (the
    reference builds its kd-tree once per point set); cell ranges are then
    computed against all the seeds.  `build_seconds` is the preparation time,
    which a per-cell timing amortises over the n seeds."""

    def __init__(self, xyz: np.ndarray, w: np.ndarray | None):
        import time
        self.x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.n = len(self.x)
        self.w = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
        t = time.perf_counter()
        self.h = port().orc_cells_prepare(_p(self.x), _p(self.w), self.n)
        self.build_seconds = time.perf_counter() - t
        if not self.h:
            raise RuntimeError("oracle prepare failed")

    def range(self, i0: int, i1: int, nthreads: int, k0: int = 20, max_nbr: int = 96) -> dict:
        """Cells [i0, i1): seconds taken, clips per cell and the results."""
        import time
        m = i1 - i0
        out = dict(vol=np.zeros(m), mg=np.zeros(3 * m), cnt=np.zeros(m, np.uint32),
                   nidx=np.zeros(m * max_nbr, np.uint32), narea=np.zeros(m * max_nbr),
                   k_list=np.zeros(m, np.uint32), n_clip=np.zeros(m, np.uint32),
                   status=np.zeros(m, np.int32))
        ne = ctypes.c_long(0)
        t = time.perf_counter()
        r = port().orc_cells_prepared_range(
            self.h, i0, i1, k0, 1, 1, nthreads, _p(out["vol"]), _p(out["mg"]), _p(out["cnt"]),
            _p(out["nidx"]), _p(out["narea"]), max_nbr, _p(out["k_list"]), _p(out["n_clip"]),
            _p(out["status"]), ctypes.byref(ne))
        out["seconds"] = time.perf_counter() - t
        if r != 0 or (out["status"] == 4).any():
            raise RuntimeError("oracle cells failed")
        out["mean_clips"] = float(out["n_clip"].mean()) if m else 0.0
        return out

    def close(self) -> None:
        if self.h:
            port().orc_cells_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cells_range_time(xyz: np.ndarray, w: np.ndarray | None, i0: int, i1: int,
                     nthreads: int, max_nbr: int = 96) -> float:
    """Seconds the CPU restatement takes for cells [i0, i1) of all the seeds,
    grid build included (the bounded CPU-baseline sample); raises if a cell
    failed."""
    import time
    t = time.perf_counter()
    pc = PreparedCells(xyz, w)
    pc.range(i0, i1, nthreads, max_nbr=max_nbr)
    pc.close()
    return time.perf_counter() - t


def ref_cells_obj(xyz: np.ndarray, w: np.ndarray | None, which, shrink: float = 0.0,
                  k0: int = 20) -> str:
    """The reference's ConvexCell::save text of the cells `which`, one after
    the other with continuing vertex numbers (reference build only)."""
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    wh = np.ascontiguousarray(which, dtype=np.uint32)
    cap = 1 << 16
    while True:
        buf = ctypes.create_string_buffer(cap)
        r = ref().ref_cells_save(_p(x), _p(wa), len(x), k0, 1, _p(wh), len(wh), shrink, buf, cap)
        if r >= 0:
            return buf.value.decode()
        cap *= 4


def ref_rvd_volume(mesh_xyz: np.ndarray, tets: np.ndarray, seeds: np.ndarray) -> dict:
    """The reference's volumetric RestrictedVoronoiDiagram of the seeds in
    the tetrahedral mesh: mass and first moment per cell (compute_centroids),
    CVT energy and gradient (compute_CVT_func_grad).  Reference build only."""
    v = np.ascontiguousarray(mesh_xyz, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(tets, dtype=np.uint32).reshape(-1, 4)
    x = np.ascontiguousarray(seeds, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    out = dict(m=np.zeros(n), mg=np.zeros((n, 3)), g=np.zeros((n, 3)))
    f = ctypes.c_double(0.0)
    r = ref().ref_rvd_volume(_p(v), len(v), _p(t), len(t), _p(x), n, _p(out["mg"]), _p(out["m"]),
                             ctypes.byref(f), _p(out["g"]))
    if r != 0:
        raise RuntimeError("ref_rvd_volume failed")
    out["f"] = f.value
    return out


def ref_cvt_newton(mesh_xyz: np.ndarray, tets: np.ndarray, seeds: np.ndarray, nb_iter: int,
                   m: int = 7) -> tuple[np.ndarray, float]:
    """The reference's CentroidalVoronoiTesselation::Newton_iterations
    (voronoi/CVT.cpp:272-307, HLBFGS) on the volumetric tet mesh: the moved
    seeds and the CVT energy there.  Reference build only."""
    v = np.ascontiguousarray(mesh_xyz, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(tets, dtype=np.uint32).reshape(-1, 4)
    x = np.array(seeds, dtype=np.float64).reshape(-1, 3)
    f = ctypes.c_double(0.0)
    r = ref().ref_cvt_newton(_p(v), len(v), _p(t), len(t), _p(x), len(x), nb_iter, m,
                             ctypes.byref(f))
    if r != 0:
        raise RuntimeError("ref_cvt_newton failed")
    return x, f.value


def ref_periodic_cells(xyz: np.ndarray, w: np.ndarray | None = None, period: float = 1.0,
                       max_nbr: int = 96) -> dict:
    """Laguerre cells in the periodic cube by the reference's
    PeriodicDelaunay3d (reference build only): vol, mg and per-cell facets
    (real index, image translation code, area) as CSR."""
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    out = dict(vol=np.zeros(n), mg=np.zeros((n, 3)), cnt=np.zeros(n, np.uint32),
               nidx=np.zeros((n, max_nbr), np.uint32), nsh=np.zeros((n, max_nbr), np.uint8),
               narea=np.zeros((n, max_nbr)))
    r = ref().ref_periodic_cells(_p(x), _p(wa), n, period, _p(out["vol"]), _p(out["mg"]),
                                 _p(out["cnt"]), _p(out["nidx"]), _p(out["nsh"]),
                                 _p(out["narea"]), max_nbr)
    if r != 0 or (out["cnt"] > max_nbr).any():
        raise RuntimeError("ref_periodic_cells failed")
    cnt = out["cnt"].astype(np.int64)
    rowptr = np.zeros(n + 1, np.int64)
    rowptr[1:] = np.cumsum(cnt)
    mask = np.arange(max_nbr)[None, :] < cnt[:, None]
    return dict(vol=out["vol"], mg=out["mg"], rowptr=rowptr, nbr=out["nidx"][mask],
                shift=out["nsh"][mask], area=out["narea"][mask])


def det4_sign(p0, p1, p2, p3) -> int:
    a = [np.ascontiguousarray(p, dtype=np.float64) for p in (p0, p1, p2, p3)]
    return int(port().orc_det4_sign(*[_p(x) for x in a]))
