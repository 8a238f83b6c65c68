"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point include/recurgreen.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

import recurgreen_gb300 as rg
from recurgreen_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(rg_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libso():
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    d = _declared()
    assert "rg_init" in d and "rg_compute_tdistrib" in d and "rg_tdistrib_batch" in d
    assert sorted(rg.EXPORTS) == d, "python binding list and header disagree"


def test_library_exports_all_declared(libso):
    missing = [n for n in _declared() if not hasattr(libso, n)]
    assert not missing, missing


def test_last_error_empty_and_bad_args(libso):
    libso.rg_last_error.restype = ctypes.c_char_p
    assert libso.rg_last_error() in (b"",)
    # NULL arguments are rejected on the host before any CUDA call.
    out = ctypes.c_void_p()
    assert libso.rg_init(None, ctypes.byref(out)) == rg.RG_ERR_INVALID_ARG
    assert b"NULL" in libso.rg_last_error()
    assert libso.rg_get_nmu(None) == -1


def test_histogram_rejects_unsorted_bins_on_host(libso):
    import numpy as np
    b = np.array([0.0, 0.5, 0.25, 1.0])
    s = np.array([0.1])
    h = np.zeros(3)
    m = ctypes.c_double()
    dp = ctypes.POINTER(ctypes.c_double)
    libso.rg_histogram.argtypes = [dp, ctypes.c_int64, dp, ctypes.c_int, dp, dp]
    rc = libso.rg_histogram(s.ctypes.data_as(dp), 1, b.ctypes.data_as(dp), 3, h.ctypes.data_as(dp), ctypes.byref(m))
    assert rc == rg.RG_ERR_INVALID_ARG
