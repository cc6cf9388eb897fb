"""GB300-native meshless Voronoi/Laguerre cell engine.

A drop-in for geogram's meshless cell path.  The Python surface mirrors the
reference's C++ one:

  NearestNeighborSearch   points/nn_search.h:69-262 (set_points,
                          get_nearest_neighbors by point or by index)
  compute_cells           the results of VBW::ConvexCell for every seed
                          (volume, compute_mg, v_global_index, facet_area;
                          voronoi/convex_cell.h:768-830), clipped until the
                          security radius certifies them (generic_RVD.h:
                          2278-2352)
  lloyd_step / lloyd_iterations
                          CentroidalVoronoiTesselation::Lloyd_iterations
                          (voronoi/CVT.cpp:133-167) on meshless cells
  ot_solve / ot_gradient_hessian
                          semi-discrete optimal transport to the uniform
                          measure on a box (exploragram OptimalTransportMap3d,
                          driven by compute_OTM/main.cpp:280-296): damped
                          Newton on the weights, the dual's gradient and
                          Laguerre Hessian
  ot_separable_start_device
                          an analytic start for it from the seeds' marginal
                          distributions (no reference counterpart)

Everything runs on the GPU through libgbv.so (C ABI in include/gbv.h).
Host arrays are numpy; device arrays are torch CUDA tensors.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (CELL_ALL_NEIGHBOURS, CELL_CERTIFIED, CELL_DUPLICATE, CELL_STALLED,
                   CERTIFY_POWER_RANGE, CERTIFY_SECURITY_RADIUS, PRECISION_FP32_GEOMETRY,
                   PRECISION_FP32_RECHECK,
                   PRECISION_FP64, CellOptions, CellReport, GbvError, OtOptions, OtReport)

__all__ = [
    "Context", "NearestNeighborSearch", "Cells", "compute_cells", "lloyd_step",
    "lloyd_iterations", "compute_cells_device", "device_results", "GbvError", "CELL_CERTIFIED", "CELL_ALL_NEIGHBOURS", "CELL_DUPLICATE",
    "CELL_STALLED",
    "PRECISION_FP64", "PRECISION_FP32_RECHECK", "PRECISION_FP32_GEOMETRY", "cell_options", "CERTIFY_SECURITY_RADIUS",
    "CERTIFY_POWER_RANGE", "ot_options", "ot_solve", "ot_solve_device", "ot_gradient_hessian",
    "ot_solve_levels", "ot_solve_levels_device", "ot_separable_start_device", "CellMesh",
    "cells_mesh", "restricted_cells", "cvt_newton", "periodic_cells",
]


class Context:
    """One GPU context (a CUDA stream plus the device buffers)."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.gbv_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def device_bytes(self) -> tuple[int, int]:
        """(bytes held now, most bytes held at once) in device memory."""
        peak = ctypes.c_uint64()
        now = self._lib.gbv_device_bytes(self.handle, ctypes.byref(peak))
        return int(now), int(peak.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.gbv_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _precision(precision: str | int) -> int:
    if isinstance(precision, str):
        return {"fp64": PRECISION_FP64, "fp32": PRECISION_FP32_RECHECK,
                "fp32_recheck": PRECISION_FP32_RECHECK,
                "fp32_geometry": PRECISION_FP32_GEOMETRY}[precision]
    return int(precision)


def cell_options(box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), k0: int = 20, check_sr: bool = True,
                 precision: str | int = "fp64", certification: str = "security_radius",
                 first_k: int = 0, predicates: str = "exact") -> CellOptions:
    o = CellOptions()
    _lib.load().gbv_cell_options_default(ctypes.byref(o))
    for c in range(3):
        o.box_min[c] = float(box[0][c])
        o.box_max[c] = float(box[1][c])
    o.k0 = int(k0)
    o.check_sr = 1 if check_sr else 0
    o.precision = _precision(precision)
    o.certification = {"security_radius": CERTIFY_SECURITY_RADIUS,
                       "power_range": CERTIFY_POWER_RANGE}[certification]
    o.first_k = int(first_k)
    o.predicates = {"exact": _lib.PREDICATES_EXACT, "fast": _lib.PREDICATES_FAST}[predicates]
    return o


def ot_options(box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), tol: float = 1e-6, max_newton: int = 100,
               max_cg: int = 4000, precision: str | int = "fp32", cg_rtol: float = 1e-4,
               step_growth: float = 4.0) -> OtOptions:
    o = OtOptions()
    _lib.load().gbv_ot_options_default(ctypes.byref(o))
    for c in range(3):
        o.box_min[c] = float(box[0][c])
        o.box_max[c] = float(box[1][c])
    o.tol = float(tol)
    o.max_newton = int(max_newton)
    o.max_cg = int(max_cg)
    o.precision = _precision(precision)
    o.cg_rtol = float(cg_rtol)
    o.step_growth = float(step_growth)
    return o


class NearestNeighborSearch:
    """GEO::NearestNeighborSearch on the GPU (points/nn_search.h:69-262).

    The reference's kd-tree stores a pointer to the caller's points
    (kd_tree.cpp:121-126); here the points are copied to the GPU by
    set_points, so the caller's array may be released afterwards.
    """

    def __init__(self, dimension: int = 3, ctx: Context | None = None):
        if dimension not in (3, 4):
            raise ValueError("dimension must be 3 or 4")
        self.dimension = dimension
        # the point set lives in the context: one context per search object
        self.ctx = ctx or Context(0)
        self.nb_points = 0

    def stride_supported(self) -> bool:
        return True

    def set_points(self, points: np.ndarray, stride: int | None = None) -> None:
        pts = np.ascontiguousarray(points, dtype=np.float64)
        if stride is None:
            pts = pts.reshape(-1, self.dimension)
            stride = self.dimension
        n = pts.size // stride
        _lib.check(self.ctx._lib.gbv_nn_set_points(self.ctx.handle, n, _lib.ptr(pts),
                                                   self.dimension, stride))
        self.nb_points = n

    def get_nearest_neighbors(self, k: int, query: np.ndarray):
        """k nearest stored points of each query row: (idx, d2), ascending."""
        q = np.ascontiguousarray(query, dtype=np.float64).reshape(-1, self.dimension)
        idx = np.empty((len(q), k), np.uint32)
        d2 = np.empty((len(q), k), np.float64)
        _lib.check(self.ctx._lib.gbv_nn_get_nearest_neighbors(
            self.ctx.handle, len(q), _lib.ptr(q), k, _lib.ptr(idx), _lib.ptr(d2)))
        return idx, d2

    def get_nearest_neighbors_by_index(self, k: int):
        """k nearest of every stored point, the point itself first (d2=0)."""
        idx = np.empty((self.nb_points, k), np.uint32)
        d2 = np.empty((self.nb_points, k), np.float64)
        _lib.check(self.ctx._lib.gbv_nn_get_nearest_neighbors_all(
            self.ctx.handle, k, _lib.ptr(idx), _lib.ptr(d2)))
        return idx, d2


@dataclass
class Cells:
    """Per-seed results, in the caller's seed order.

    volume[i]   ConvexCell::volume()
    mg[i]       ConvexCell::compute_mg() (volume-weighted centroid)
    rowptr, neighbors, facet_area: CSR of the facets shared with other
                seeds, v_global_index(v) and facet_area(v) in the
                reference's order (clipping order)
    status[i]   CELL_CERTIFIED / CELL_ALL_NEIGHBOURS / CELL_DUPLICATE
    """
    volume: np.ndarray
    mg: np.ndarray
    rowptr: np.ndarray
    neighbors: np.ndarray
    facet_area: np.ndarray
    status: np.ndarray
    report: dict = field(default_factory=dict)

    def barycenter(self) -> np.ndarray:
        """ConvexCell::barycenter (convex_cell.cpp:1255-1265): mg/m, 0-safe."""
        m = self.volume[:, None]
        return np.where(m != 0.0, self.mg / np.where(m != 0.0, m, 1.0), self.mg)

    def neighbors_of(self, i: int):
        a, b = self.rowptr[i], self.rowptr[i + 1]
        return self.neighbors[a:b], self.facet_area[a:b]


def compute_cells(xyz: np.ndarray, weights: np.ndarray | None = None, *,
                  box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), k0: int = 20, check_sr: bool = True,
                  precision: str | int = "fp64", certification: str = "security_radius",
                  first_k: int = 0, predicates: str = "exact", ctx: Context | None = None) -> Cells:
    """Certified Laguerre cells of the seeds xyz (n x 3) with weights (n).

    certification "security_radius" reproduces the reference's clipping
    loop; "power_range" finds every seed that can cut a cell by a range
    query on the power distance (for widely spread weights).  first_k: the
    first kNN list length of the security-radius loop (0: automatic); the
    cells do not depend on it.  predicates "fast": the reference's
    use_exact_predicates(false) (FP64 det4x4, conflict iff > 0)."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64).reshape(n)
    o = cell_options(box, k0, check_sr, precision, certification, first_k, predicates)
    rep = CellReport()
    L = ctx._lib
    _lib.check(L.gbv_cells_compute(ctx.handle, _lib.ptr(x), _lib.ptr(w), n, ctypes.byref(o),
                                   ctypes.byref(rep)))
    vol = np.empty(n)
    mg = np.empty((n, 3))
    rowptr = np.empty(n + 1, np.uint32)
    nbr = np.empty(max(rep.nnz, 1), np.uint32)
    area = np.empty(max(rep.nnz, 1))
    status = np.empty(n, np.int32)
    _lib.check(L.gbv_cells_fetch(ctx.handle, _lib.ptr(vol), _lib.ptr(mg), _lib.ptr(rowptr),
                                 _lib.ptr(nbr), _lib.ptr(area), _lib.ptr(status)))
    ctx.last_n, ctx.last_nnz = n, rep.nnz
    return Cells(vol, mg, rowptr, nbr[:rep.nnz], area[:rep.nnz], status, rep.as_dict())


@dataclass
class CellMesh:
    """Polytopes of cells (ConvexCell::save / append_to_mesh,
    voronoi/convex_cell.cpp:282-352, 371-444), cell after cell.

    cells[k]             original index of the k-th exported cell
    vertices             corners (x, y, z), in each cell's valid-list order
    cell_vertex_ptr      cell k owns vertices[cell_vertex_ptr[k]:cell_vertex_ptr[k+1]]
    cell_face_ptr        ... and polygons cell_face_ptr[k]:cell_face_ptr[k+1]
    face_ptr, face_vertices
                         polygon f is face_vertices[face_ptr[f]:face_ptr[f+1]],
                         corner numbers local to its cell
    face_seed[f]         the seed across polygon f (v_global_index), or
                         0xFFFFFFFF for a box face
    """
    cells: np.ndarray
    vertices: np.ndarray
    cell_vertex_ptr: np.ndarray
    cell_face_ptr: np.ndarray
    face_ptr: np.ndarray
    face_vertices: np.ndarray
    face_seed: np.ndarray

    def obj_text(self, v_offset: int = 1, shrink: float = 0.0,
                 barycenters: np.ndarray | None = None) -> str:
        """The cells as ConvexCell::save writes them one after the other
        ("v x y z" lines, then "f i j k ..." lines, vertex numbers from
        v_offset and continuing across cells); shrink moves every corner
        toward its cell's barycenter (mg / m, one row per exported cell)
        as p = shrink g + (1 - shrink) p."""
        if shrink != 0.0 and barycenters is None:
            raise ValueError("shrink needs the cells' barycenters")
        out = []
        off = v_offset
        for k in range(len(self.cells)):
            v0, v1 = int(self.cell_vertex_ptr[k]), int(self.cell_vertex_ptr[k + 1])
            g = barycenters[k] if shrink != 0.0 else None
            for p in self.vertices[v0:v1]:
                x, y, z = float(p[0]), float(p[1]), float(p[2])
                if g is not None:
                    x = shrink * float(g[0]) + (1.0 - shrink) * x
                    y = shrink * float(g[1]) + (1.0 - shrink) * y
                    z = shrink * float(g[2]) + (1.0 - shrink) * z
                out.append("v %g %g %g\n" % (x, y, z))
            for f in range(int(self.cell_face_ptr[k]), int(self.cell_face_ptr[k + 1])):
                ids = self.face_vertices[self.face_ptr[f]:self.face_ptr[f + 1]]
                out.append("f " + "".join(f"{int(i) + off} " for i in ids) + "\n")
            off += v1 - v0
        return "".join(out)

    def save_obj(self, path: str, **kw) -> None:
        with open(path, "w") as f:
            f.write(self.obj_text(**kw))


def cells_mesh(cells=None, ctx: Context | None = None) -> CellMesh:
    """Polytopes of cells of the last compute on ctx (all cells when None)."""
    ctx = ctx or default_context()
    L = ctx._lib
    if cells is None:
        ci = None
        m = int(getattr(ctx, "last_n", 0))
    else:
        ci = np.ascontiguousarray(cells, dtype=np.uint32).reshape(-1)
        m = len(ci)
    sz = _lib.MeshSizes()
    _lib.check(L.gbv_cells_mesh(ctx.handle, _lib.ptr(ci), m, ctypes.byref(sz), None, None, None,
                                None, None, None))
    nv, nf = int(sz.n_vertices), int(sz.n_faces)
    out = CellMesh(cells=ci if ci is not None else np.arange(m, dtype=np.uint32),
                   vertices=np.empty((nv, 3)), cell_vertex_ptr=np.empty(m + 1, np.uint32),
                   cell_face_ptr=np.empty(m + 1, np.uint32), face_ptr=np.empty(nf + 1, np.uint32),
                   face_vertices=np.empty(3 * nv, np.uint32), face_seed=np.empty(nf, np.uint32))
    _lib.check(L.gbv_cells_mesh(ctx.handle, _lib.ptr(ci), m, ctypes.byref(sz),
                                _lib.ptr(out.vertices), _lib.ptr(out.cell_vertex_ptr),
                                _lib.ptr(out.cell_face_ptr), _lib.ptr(out.face_ptr),
                                _lib.ptr(out.face_vertices), _lib.ptr(out.face_seed)))
    return out


def periodic_cells(xyz: np.ndarray, weights: np.ndarray | None = None, *, period: float = 1.0,
                   k0: int = 20, precision="fp64", ctx: Context | None = None) -> dict:
    """Laguerre cells in the periodic cube [0, period)^3 (the reference's
    PeriodicDelaunay3d + copy_Laguerre_cell_from_Delaunay,
    delaunay/periodic_delaunay_3d.cpp:3634-3734): volume, mg, and per
    facet the seed across it, its image translation code shift =
    (tx+1)*9 + (ty+1)*3 + (tz+1) (13: none) and the facet area (CSR)."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64).reshape(n)
    o = cell_options(k0=k0, precision=precision)
    rep = CellReport()
    L = ctx._lib
    _lib.check(L.gbv_periodic_cells(ctx.handle, _lib.ptr(x), _lib.ptr(w), n, float(period),
                                    ctypes.byref(o), ctypes.byref(rep)))
    k = max(rep.nnz, 1)
    out = dict(volume=np.empty(n), mg=np.empty((n, 3)), rowptr=np.empty(n + 1, np.uint32),
               neighbors=np.empty(k, np.uint32), shift=np.empty(k, np.uint8),
               facet_area=np.empty(k))
    _lib.check(L.gbv_periodic_fetch(ctx.handle, _lib.ptr(out["volume"]), _lib.ptr(out["mg"]),
                                    _lib.ptr(out["rowptr"]), _lib.ptr(out["neighbors"]),
                                    _lib.ptr(out["shift"]), _lib.ptr(out["facet_area"])))
    for key in ("neighbors", "shift", "facet_area"):
        out[key] = out[key][:rep.nnz]
    out["report"] = rep.as_dict()
    return out


def restricted_cells(mesh_xyz: np.ndarray, tets: np.ndarray, xyz: np.ndarray,
                     weights: np.ndarray | None = None, *, k0: int = 20, precision="fp64",
                     ctx: Context | None = None) -> dict:
    """Cells of the seeds restricted to a tetrahedral mesh (the reference's
    volumetric RestrictedVoronoiDiagram, voronoi/RVD.cpp:429-530 and
    :792-910): per seed the mass m and first moment mg of its cell inside the
    mesh, the CVT energy f = sum_i int |x - p_i|^2 and its gradient g."""
    ctx = ctx or default_context()
    v = np.ascontiguousarray(mesh_xyz, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(tets, dtype=np.uint32).reshape(-1, 4)
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64).reshape(n)
    o = cell_options(k0=k0, precision=precision)
    rep = CellReport()
    out = dict(m=np.empty(n), mg=np.empty((n, 3)), g=np.empty((n, 3)))
    f = ctypes.c_double(0.0)
    _lib.check(ctx._lib.gbv_restricted_cells(ctx.handle, _lib.ptr(v), len(v), _lib.ptr(t), len(t),
                                             _lib.ptr(x), _lib.ptr(w), n, ctypes.byref(o),
                                             _lib.ptr(out["m"]), _lib.ptr(out["mg"]),
                                             ctypes.byref(f), _lib.ptr(out["g"]),
                                             ctypes.byref(rep)))
    out["f"] = f.value
    out["report"] = rep.as_dict()
    ctx.last_n, ctx.last_nnz = n, rep.nnz
    return out


def cvt_newton(mesh_xyz: np.ndarray, tets: np.ndarray, xyz: np.ndarray, nb_iter: int, *,
               m: int = 7, k0: int = 20, precision="fp64",
               ctx: Context | None = None) -> tuple[np.ndarray, np.ndarray]:
    """CentroidalVoronoiTesselation::Newton_iterations (voronoi/CVT.cpp:
    272-307) on a tetrahedral mesh: L-BFGS with m pairs on the restricted
    cells' CVT energy and gradient, nb_iter + 1 steps as the reference's
    HLBFGS takes.  Returns the moved seeds and the energy at the start and
    after each step."""
    ctx = ctx or default_context()
    v = np.ascontiguousarray(mesh_xyz, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(tets, dtype=np.uint32).reshape(-1, 4)
    x = np.array(xyz, dtype=np.float64).reshape(-1, 3)
    o = cell_options(k0=k0, precision=precision)
    energy = np.zeros(nb_iter + 2)
    its = ctypes.c_uint32(0)
    _lib.check(ctx._lib.gbv_cvt_newton(ctx.handle, _lib.ptr(v), len(v), _lib.ptr(t), len(t),
                                       _lib.ptr(x), len(x), ctypes.byref(o), nb_iter, m,
                                       _lib.ptr(energy), ctypes.byref(its)))
    return x, energy[:its.value + 1]


def _dev_arg(t, name: str, n: int | None = None, cols: int | None = None,
             ctx: Context | None = None):
    """A device argument as the C ABI reads it: a contiguous float64 CUDA
    tensor on the context's device, n x cols (cols given) or n (cols None);
    None passes through.  The entry points get raw pointers, so anything
    else would be misread (another GPU's tensor would be read without peer
    access)."""
    if t is None:
        return None
    if not (getattr(t, "is_cuda", False) and str(t.dtype) == "torch.float64"
            and t.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous float64 CUDA tensor")
    if ctx is not None and t.device.index != ctx.device:
        raise ValueError(f"{name} is on cuda:{t.device.index}, the context on cuda:{ctx.device}")
    shape = tuple(t.shape)
    want_dim = 1 if cols is None else 2
    if len(shape) != want_dim or (cols is not None and shape[1] != cols) or \
            (n is not None and shape[0] != n):
        raise ValueError(f"{name} has shape {shape}, expected "
                         f"{(n if n is not None else 'n',) + (() if cols is None else (cols,))}")
    return t


def compute_cells_device(xyz, weights=None, *, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
                         k0: int = 20, check_sr: bool = True, precision="fp64",
                         certification: str = "security_radius", first_k: int = 0,
                         stream=None, ctx: Context | None = None) -> dict:
    """Same on torch CUDA tensors (float64, n x 3 and n); results stay on
    the device (read them with device_results)."""
    ctx = ctx or default_context()
    n = _dev_arg(xyz, "xyz", cols=3, ctx=ctx).shape[0]
    _dev_arg(weights, "weights", n, ctx=ctx)
    o = cell_options(box, k0, check_sr, precision, certification, first_k)
    rep = CellReport()
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    _lib.check(ctx._lib.gbv_cells_compute_device(ctx.handle, _lib.ptr(xyz), _lib.ptr(weights), n,
                                                 ctypes.byref(o), st, ctypes.byref(rep)))
    ctx.last_n, ctx.last_nnz = n, rep.nnz
    return rep.as_dict()


def device_results(ctx: Context | None = None) -> dict:
    """Copies the results of the last compute on `ctx` to host arrays."""
    ctx = ctx or default_context()
    n, nnz = ctx.last_n, ctx.last_nnz
    out = dict(volume=np.empty(n), mg=np.empty((n, 3)), rowptr=np.empty(n + 1, np.uint32),
               neighbors=np.empty(max(nnz, 1), np.uint32), facet_area=np.empty(max(nnz, 1)),
               status=np.empty(n, np.int32))
    _lib.check(ctx._lib.gbv_cells_fetch(ctx.handle, _lib.ptr(out["volume"]), _lib.ptr(out["mg"]),
                                        _lib.ptr(out["rowptr"]), _lib.ptr(out["neighbors"]),
                                        _lib.ptr(out["facet_area"]), _lib.ptr(out["status"])))
    out["neighbors"] = out["neighbors"][:nnz]
    out["facet_area"] = out["facet_area"][:nnz]
    return out


def lloyd_step(xyz: np.ndarray, weights: np.ndarray | None = None, *,
               box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), precision="fp64",
               ctx: Context | None = None) -> tuple[np.ndarray, dict]:
    """One Lloyd iteration (CVT.cpp:133-167): returns the moved seeds."""
    ctx = ctx or default_context()
    x = np.array(xyz, dtype=np.float64, copy=True).reshape(-1, 3)
    n = len(x)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64).reshape(n)
    o = cell_options(box, 20, True, precision)
    rep = CellReport()
    _lib.check(ctx._lib.gbv_lloyd_step(ctx.handle, _lib.ptr(x), _lib.ptr(w), n, ctypes.byref(o),
                                       ctypes.byref(rep)))
    return x, rep.as_dict()


def lloyd_iterations(xyz_dev, iters: int, weights_dev=None, *,
                     box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), precision="fp64", stream=None,
                     ctx: Context | None = None) -> dict:
    """`iters` Lloyd iterations in place on a torch CUDA tensor (n x 3)."""
    ctx = ctx or default_context()
    n = _dev_arg(xyz_dev, "xyz_dev", cols=3, ctx=ctx).shape[0]
    _dev_arg(weights_dev, "weights_dev", n, ctx=ctx)
    o = cell_options(box, 20, True, precision)
    rep = CellReport()
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    _lib.check(ctx._lib.gbv_lloyd_device(ctx.handle, _lib.ptr(xyz_dev), _lib.ptr(weights_dev),
                                         xyz_dev.shape[0], iters, ctypes.byref(o), st,
                                         ctypes.byref(rep)))
    return rep.as_dict()


def ot_solve(xyz: np.ndarray, nu: np.ndarray | None = None, w0: np.ndarray | None = None, *,
             box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), tol: float = 1e-6, max_newton: int = 100,
             max_cg: int = 4000, precision="fp32", cg_rtol: float = 1e-4,
             step_growth: float = 4.0, ctx: Context | None = None
             ) -> tuple[np.ndarray, dict]:
    """Weights of the seeds whose Laguerre cells in the box have volumes nu
    (default: box volume / n each), starting from w0 (default zeros)."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    w = np.zeros(n) if w0 is None else np.array(w0, dtype=np.float64, copy=True).reshape(n)
    m = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64).reshape(n)
    o = ot_options(box, tol, max_newton, max_cg, precision, cg_rtol, step_growth)
    rep = OtReport()
    _lib.check(ctx._lib.gbv_ot_solve(ctx.handle, _lib.ptr(x), _lib.ptr(m), n, ctypes.byref(o),
                                     _lib.ptr(w), ctypes.byref(rep)))
    return w, rep.as_dict()


def ot_solve_device(xyz_dev, w_dev, nu_dev=None, *, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
                    tol: float = 1e-6, max_newton: int = 100, max_cg: int = 4000,
                    precision="fp32", cg_rtol: float = 1e-4, step_growth: float = 4.0,
                    stream=None, ctx: Context | None = None) -> dict:
    """ot_solve on torch CUDA tensors; w_dev (float64, n) is updated in place."""
    ctx = ctx or default_context()
    n = _dev_arg(xyz_dev, "xyz_dev", cols=3, ctx=ctx).shape[0]
    _dev_arg(w_dev, "w_dev", n, ctx=ctx)
    _dev_arg(nu_dev, "nu_dev", n, ctx=ctx)
    o = ot_options(box, tol, max_newton, max_cg, precision, cg_rtol, step_growth)
    rep = OtReport()
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    _lib.check(ctx._lib.gbv_ot_solve_device(ctx.handle, _lib.ptr(xyz_dev), _lib.ptr(nu_dev),
                                            xyz_dev.shape[0], ctypes.byref(o), _lib.ptr(w_dev),
                                            st, ctypes.byref(rep)))
    return rep.as_dict()


def ot_separable_start_device(xyz_dev, *, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), stream=None,
                              ctx: Context | None = None):
    """Starting weights for ot_solve_device from the seeds' marginal
    distributions (float64 tensor, n; not centred): w = |p|^2 - 2 sum_a
    Phi_a(p_a), Phi_a' the piecewise-linear CDF of axis a.  No cell of these
    weights is empty for distinct seeds.  xyz_dev: float64 CUDA tensor, n x 3."""
    import torch
    ctx = ctx or default_context()
    x = _dev_arg(xyz_dev, "xyz_dev", cols=3, ctx=ctx)
    w = torch.empty(x.shape[0], dtype=torch.float64, device=x.device)
    o = ot_options(box)
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    _lib.check(ctx._lib.gbv_ot_separable_start(ctx.handle, _lib.ptr(x), x.shape[0],
                                               ctypes.byref(o), _lib.ptr(w), st))
    return w


def ot_gradient_hessian(xyz: np.ndarray, w: np.ndarray, nu: np.ndarray | None = None, *,
                        box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), precision="fp32",
                        ctx: Context | None = None):
    """Gradient nu - vol and CSR Hessian (rowptr, col, val, diag) of the dual."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    ww = np.ascontiguousarray(w, dtype=np.float64).reshape(n)
    m = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64).reshape(n)
    o = ot_options(box, precision=precision)
    nnz = ctypes.c_uint64()
    L = ctx._lib
    _lib.check(L.gbv_ot_gradient_hessian(ctx.handle, _lib.ptr(x), _lib.ptr(ww), _lib.ptr(m), n,
                                         ctypes.byref(o), None, None, None, None, None, 0,
                                         ctypes.byref(nnz)))
    k = max(nnz.value, 1)
    g = np.empty(n)
    rp = np.empty(n + 1, np.uint32)
    col = np.empty(k, np.uint32)
    val = np.empty(k)
    diag = np.empty(n)
    _lib.check(L.gbv_ot_gradient_hessian(ctx.handle, _lib.ptr(x), _lib.ptr(ww), _lib.ptr(m), n,
                                         ctypes.byref(o), _lib.ptr(g), _lib.ptr(rp),
                                         _lib.ptr(col), _lib.ptr(val), _lib.ptr(diag), k,
                                         ctypes.byref(nnz)))
    return g, (rp, col[:nnz.value], val[:nnz.value], diag)


def ot_solve_levels(xyz: np.ndarray, nu: np.ndarray | None = None, *, ratio: int = 8,
                    min_level: int = 20000, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
                    tol: float = 1e-6, max_newton: int = 100, precision="fp32",
                    ctx: Context | None = None) -> tuple[np.ndarray, dict]:
    """Multilevel solve (optimize_levels of the reference's compute_OTM): nested
    random subsets of n / ratio^l seeds, coarse to fine, each starting from
    the coarser weights interpolated at its seeds."""
    ctx = ctx or default_context()
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(x)
    w = np.zeros(n)
    m = None if nu is None else np.ascontiguousarray(nu, dtype=np.float64).reshape(n)
    o = ot_options(box, tol, max_newton, precision=precision)
    rep = OtReport()
    _lib.check(ctx._lib.gbv_ot_solve_levels(ctx.handle, _lib.ptr(x), _lib.ptr(m), n,
                                            ctypes.byref(o), int(ratio), int(min_level),
                                            _lib.ptr(w), ctypes.byref(rep)))
    return w, rep.as_dict()


def ot_solve_levels_device(xyz_dev, w_dev, nu_dev=None, *, ratio: int = 8,
                           min_level: int = 20000, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)),
                           tol: float = 1e-6, max_newton: int = 100, precision="fp32",
                           stream=None, ctx: Context | None = None) -> dict:
    """ot_solve_levels on torch CUDA tensors; w_dev (float64, n) receives the weights."""
    ctx = ctx or default_context()
    n = _dev_arg(xyz_dev, "xyz_dev", cols=3, ctx=ctx).shape[0]
    _dev_arg(w_dev, "w_dev", n, ctx=ctx)
    _dev_arg(nu_dev, "nu_dev", n, ctx=ctx)
    o = ot_options(box, tol, max_newton, precision=precision)
    rep = OtReport()
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    _lib.check(ctx._lib.gbv_ot_solve_levels_device(ctx.handle, _lib.ptr(xyz_dev),
                                                   _lib.ptr(nu_dev), xyz_dev.shape[0],
                                                   ctypes.byref(o), int(ratio), int(min_level),
                                                   _lib.ptr(w_dev), st, ctypes.byref(rep)))
    return rep.as_dict()
