"""The tensor-core complex product (rg_ozaki_zgemm) against its exact
integer model (bit for bit) and against an extended-precision product
(FP64-level accuracy)."""
import numpy as np
import pytest

import ozaki_model as OZ
import recurgreen_gb300 as rg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M", [1, 16, 37, 100, 256, 512])
def test_ozaki_zgemm_bit_exact_against_model(M):
    rng = np.random.default_rng(100 + M)
    A = (rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))) * np.exp(rng.uniform(-20, 5, (M, 1)))
    B = (rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))) * np.exp(rng.uniform(-40, 0, (1, M)))
    if M > 3:
        A[2, :] = 0.0
        B[:, 1] = 0.0
    C = rg.ozaki_zgemm(A, B)
    ref = OZ.zgemm(A, B)
    np.testing.assert_array_equal(C.real, ref.real)
    np.testing.assert_array_equal(C.imag, ref.imag)
    ex = A.astype(np.clongdouble) @ B.astype(np.clongdouble)
    e_oz = float(np.linalg.norm(C - ex) / np.linalg.norm(ex))
    e_64 = float(np.linalg.norm(A @ B - ex) / np.linalg.norm(ex))
    assert e_oz <= max(4 * e_64, 4e-16)


def test_ozaki_zgemm_rejects_bad_sizes():
    L = rg.lib()
    z = np.zeros(4)
    for M in (0, 513):
        assert L.rg_ozaki_zgemm(M, z.ctypes.data, z.ctypes.data, z.ctypes.data) == rg.RG_ERR_INVALID_ARG
