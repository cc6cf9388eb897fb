"""ctypes binding of libgbv.so (the C ABI declared in include/gbv.h).

The library is loaded from the package directory.  There is no fallback:
if libgbv.so is missing or does not load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbv.so")

GBV_OK = 0
STATUS_NAMES = {
    0: "GBV_OK", 1: "GBV_ERR_INVALID_ARGUMENT", 2: "GBV_ERR_CUDA", 3: "GBV_ERR_NO_DEVICE",
    4: "GBV_ERR_CAPACITY", 5: "GBV_ERR_NOT_CONVERGED", 6: "GBV_ERR_STATE",
}

CELL_CERTIFIED = 0
CELL_ALL_NEIGHBOURS = 1
CELL_DUPLICATE = 2
CELL_STALLED = 3

PRECISION_FP64 = 0
PRECISION_FP32_RECHECK = 1
PRECISION_FP32_GEOMETRY = 2


class GbvError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class CellOptions(ctypes.Structure):
    _fields_ = [
        ("box_min", ctypes.c_double * 3),
        ("box_max", ctypes.c_double * 3),
        ("k0", ctypes.c_uint32),
        ("check_sr", ctypes.c_uint32),
        ("precision", ctypes.c_uint32),
        ("certification", ctypes.c_uint32),
        ("first_k", ctypes.c_uint32),
        ("predicates", ctypes.c_uint32),
    ]


CERTIFY_SECURITY_RADIUS = 0
CERTIFY_POWER_RANGE = 1

PREDICATES_EXACT = 0
PREDICATES_FAST = 1


class OtOptions(ctypes.Structure):
    _fields_ = [
        ("box_min", ctypes.c_double * 3),
        ("box_max", ctypes.c_double * 3),
        ("tol", ctypes.c_double),
        ("max_newton", ctypes.c_uint32),
        ("max_cg", ctypes.c_uint32),
        ("precision", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("cg_rtol", ctypes.c_double),
        ("step_growth", ctypes.c_double),
    ]


class OtReport(ctypes.Structure):
    _fields_ = [
        ("converged", ctypes.c_uint32),
        ("newton_iters", ctypes.c_uint32),
        ("cg_iters", ctypes.c_uint32),
        ("halvings", ctypes.c_uint32),
        ("cell_calls", ctypes.c_uint32),
        ("levels", ctypes.c_uint32),
        ("mass_error_inf", ctypes.c_double),
        ("mass_error_l2", ctypes.c_double),
        ("min_volume", ctypes.c_double),
        ("ms_total", ctypes.c_double),
        ("ms_cells", ctypes.c_double),
        ("ms_linear", ctypes.c_double),
        ("start_scale", ctypes.c_double),
        ("ms_start", ctypes.c_double),
        ("start_cg_iters", ctypes.c_uint32),
        ("reserved2", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class CellReport(ctypes.Structure):
    _fields_ = [
        ("nnz", ctypes.c_uint64),
        ("n_cells", ctypes.c_uint32),
        ("n_recheck_fp64", ctypes.c_uint32),
        ("n_more_k", ctypes.c_uint32),
        ("n_overflow", ctypes.c_uint32),
        ("max_clips", ctypes.c_uint32),
        ("knn_k", ctypes.c_uint32),
        ("mean_clips", ctypes.c_double),
        ("volume_sum", ctypes.c_double),
        ("n_exact", ctypes.c_uint64),
        ("ms_grid", ctypes.c_double),
        ("ms_knn", ctypes.c_double),
        ("ms_clip", ctypes.c_double),
        ("ms_retry", ctypes.c_double),
        ("ms_total", ctypes.c_double),
        ("n_huge", ctypes.c_uint32),
        ("n_knn_exact", ctypes.c_uint32),
        ("n_conflict_tests", ctypes.c_uint64),
        ("n_corners_created", ctypes.c_uint64),
        ("ms_clip_kernel", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class MeshSizes(ctypes.Structure):
    _fields_ = [
        ("n_vertices", ctypes.c_uint64),
        ("n_faces", ctypes.c_uint64),
        ("n_face_vertices", ctypes.c_uint64),
    ]


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32

# name -> (restype, argtypes); every function declared in include/gbv.h
SIGNATURES = {
    "gbv_last_error": (ctypes.c_char_p, []),
    "gbv_kernel_launches": (ctypes.c_uint64, []),
    "gbv_device_bytes": (ctypes.c_uint64, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "gbv_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "gbv_destroy": (ctypes.c_int, [_P]),
    "gbv_cell_options_default": (None, [ctypes.POINTER(CellOptions)]),
    "gbv_nn_set_points": (ctypes.c_int, [_P, _U32, _P, _U32, _U32]),
    "gbv_nn_get_nearest_neighbors": (ctypes.c_int, [_P, _U32, _P, _U32, _P, _P]),
    "gbv_nn_get_nearest_neighbors_all": (ctypes.c_int, [_P, _U32, _P, _P]),
    "gbv_cells_compute": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(CellOptions),
                                         ctypes.POINTER(CellReport)]),
    "gbv_cells_compute_device": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(CellOptions),
                                                _P, ctypes.POINTER(CellReport)]),
    "gbv_cells_fetch": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "gbv_cells_device_results": (ctypes.c_int, [_P] + [ctypes.POINTER(_P)] * 6),
    "gbv_lloyd_step": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(CellOptions),
                                      ctypes.POINTER(CellReport)]),
    "gbv_lloyd_device": (ctypes.c_int, [_P, _P, _P, _U32, _U32, ctypes.POINTER(CellOptions), _P,
                                        ctypes.POINTER(CellReport)]),
    "gbv_ot_options_default": (None, [ctypes.POINTER(OtOptions)]),
    "gbv_ot_solve": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(OtOptions), _P,
                                    ctypes.POINTER(OtReport)]),
    "gbv_ot_solve_device": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(OtOptions), _P, _P,
                                           ctypes.POINTER(OtReport)]),
    "gbv_ot_solve_levels": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(OtOptions), _U32,
                                           _U32, _P, ctypes.POINTER(OtReport)]),
    "gbv_ot_solve_levels_device": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(OtOptions),
                                                  _U32, _U32, _P, _P,
                                                  ctypes.POINTER(OtReport)]),
    "gbv_ot_gradient_hessian": (ctypes.c_int, [_P, _P, _P, _P, _U32, ctypes.POINTER(OtOptions),
                                               _P, _P, _P, _P, _P, ctypes.c_uint64,
                                               ctypes.POINTER(ctypes.c_uint64)]),
    "gbv_mlp_features": (ctypes.c_int, [_P, _P, _U32, _P, _P]),
    "gbv_mlp_forward": (ctypes.c_int, [_P, _P, _P, _P, _U32, _P, _P]),
    "gbv_mlp_loss_grad": (ctypes.c_int, [_P, _P, _P, _P, _P, _U32, _P,
                                         ctypes.POINTER(ctypes.c_double), _P]),
    "gbv_mlp_adam": (ctypes.c_int, [_P, _P, _P, _P, _P, _U32, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, _P]),
    "gbv_ot_warm_start": (ctypes.c_int, [_P, _P, _U32, ctypes.POINTER(OtOptions), _P, _P, _P,
                                         _P]),
    "gbv_ot_solve_learned_device": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.POINTER(OtOptions),
                                                   _P, _P, _P, _P, ctypes.POINTER(OtReport)]),
    "gbv_ot_separable_start": (ctypes.c_int, [_P, _P, _U32, ctypes.POINTER(OtOptions), _P, _P]),
    "gbv_mlp_gemm_nt": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
    "gbv_periodic_cells": (ctypes.c_int, [_P, _P, _P, _U32, ctypes.c_double,
                                          ctypes.POINTER(CellOptions), ctypes.POINTER(CellReport)]),
    "gbv_periodic_fetch": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "gbv_restricted_cells": (ctypes.c_int, [_P, _P, _U32, _P, _U32, _P, _P, _U32,
                                            ctypes.POINTER(CellOptions), _P, _P,
                                            ctypes.POINTER(ctypes.c_double), _P,
                                            ctypes.POINTER(CellReport)]),
    "gbv_cvt_newton": (ctypes.c_int, [_P, _P, _U32, _P, _U32, _P, _U32,
                                      ctypes.POINTER(CellOptions), _U32, _U32, _P,
                                      ctypes.POINTER(ctypes.c_uint32)]),
    "gbv_cells_mesh": (ctypes.c_int, [_P, _P, _U32, ctypes.POINTER(MeshSizes), _P, _P, _P, _P,
                                      _P, _P]),
    "gbv_knn_noalloc": (ctypes.c_int, [_P, _U32, _U32, _U32, _U32, _P, _P, _P]),
}

MLP_INPUTS = 19
MLP_PARAMS = 37377
MLP_NORM = 40
MLP_MAX_BATCH = 65536

_lib = None
_lock = threading.Lock()


def load() -> ctypes.CDLL:
    """Loads libgbv.so and binds every entry point (raises if missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != GBV_OK:
        msg = load().gbv_last_error()
        raise GbvError(status, msg.decode() if msg else "")


def ptr(a) -> ctypes.c_void_p:
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)
