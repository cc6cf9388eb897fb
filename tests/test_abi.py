"""The C ABI library: it loads and exports every entry point include/gbv.h
declares (no GPU needed), and the package fails loudly without a device."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gbv.h")
LIB = os.path.join(ROOT, "geogram_gb300", "libgbv.so")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbv_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from geogram_gb300 import _build
        _build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gbv_cells_compute" in names and "gbv_nn_set_points" in names
    assert len(names) >= 14


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from geogram_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_options_default(lib):
    from geogram_gb300 import _lib
    L = _lib.load()
    o = _lib.CellOptions()
    L.gbv_cell_options_default(ctypes.byref(o))
    assert (o.k0, o.check_sr, o.precision) == (20, 1, 0)
    assert list(o.box_min) == [0.0, 0.0, 0.0] and list(o.box_max) == [1.0, 1.0, 1.0]


def test_no_device_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import geogram_gb300 as g
    with pytest.raises(g.GbvError) as e:
        g.Context(0)
    assert e.value.status == 3  # GBV_ERR_NO_DEVICE


# entry points that take no context first (or report through another channel)
NO_CONTEXT = {"gbv_last_error", "gbv_kernel_launches", "gbv_device_bytes", "gbv_create",
              "gbv_destroy", "gbv_cell_options_default", "gbv_ot_options_default",
              "gbv_knn_noalloc"}


def test_null_context_is_an_argument_error(lib):
    """Every entry point that takes a context rejects NULL with
    GBV_ERR_INVALID_ARGUMENT and a message, before touching a device."""
    from geogram_gb300 import _lib
    L = _lib.load()
    checked = 0
    for name, (_, argtypes) in _lib.SIGNATURES.items():
        if name in NO_CONTEXT:
            continue
        args = [None if (t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, ctypes._Pointer))
                else t(0) for t in argtypes]
        assert getattr(L, name)(*args) == 1, name
        assert L.gbv_last_error(), name
        checked += 1
    assert checked >= 20
