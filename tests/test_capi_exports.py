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


def test_zgemm_workspace_size_follows_the_digit_layout(libso):
    """rg_zgemm_workspace_bytes (host arithmetic, no GPU): per product, both
    operands' digit planes -- 2 parts x 6 slices of FP16 digits, i.e. 24 bytes
    per entry of each operand, in 16 x 16 tiles -- and the row and column
    exponents (16-byte padded); -1 outside 1 <= M <= 512."""
    f = libso.rg_zgemm_workspace_bytes
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_int]

    def expected(M, nbatch):
        T = (M + 15) // 16
        operand = 2 * 6 * T * T * 32 * 16  # uint4 per lane per tile per plane
        exps = (2 * T * 16 * 4 + 15) // 16 * 16
        return nbatch * (2 * operand + exps)

    for M, nb in ((1, 1), (64, 5), (100, 2), (128, 3), (512, 1)):
        assert f(M, nb) == expected(M, nb), M
    assert expected(128, 1) == 2 * 24 * 128 * 128 + 1024
    assert f(0, 1) == -1 and f(513, 1) == -1 and f(16, -1) == -1
