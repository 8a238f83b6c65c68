"""The exact integer model of the tensor-core complex product (CPU): its
accuracy against an extended-precision product is that of an FP64 product,
and its level sums stay below 2^24 (checked inside the model)."""
import numpy as np
import pytest

import ozaki_model as OZ


def _case(M, rng, graded=True):
    A = rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))
    B = rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))
    if graded:  # rows of A and columns of B spread over many octaves
        A *= np.exp(rng.uniform(-20, 5, (M, 1)))
        B *= np.exp(rng.uniform(-40, 0, (1, M)))
    return A, B


@pytest.mark.parametrize("M", [1, 16, 37, 100, 256])
def test_model_accuracy_matches_fp64(M):
    rng = np.random.default_rng(M)
    for graded in (False, True):
        A, B = _case(M, rng, graded)
        ex = A.astype(np.clongdouble) @ B.astype(np.clongdouble)
        oz = OZ.zgemm(A, B)
        f64 = A @ B
        nrm = np.linalg.norm(ex)
        e_oz = float(np.linalg.norm(oz - ex) / nrm)
        e_64 = float(np.linalg.norm(f64 - ex) / nrm)
        # normwise: within a few units of an FP64 product's own error
        assert e_oz <= max(4 * e_64, 4e-16), (M, graded, e_oz, e_64)
        # elementwise against |A||B| (the FP64 product's error bound, K eps |A||B|)
        den = np.abs(A) @ np.abs(B)
        assert float(np.max(np.abs(oz - ex) / den)) <= M * 2.0 ** -53


def test_model_zero_rows_and_extremes():
    M = 20
    rng = np.random.default_rng(3)
    A, B = _case(M, rng)
    A[3, :] = 0.0
    B[:, 5] = 0.0
    A[7, 2] = 1e-310  # subnormal entries count as zero digits
    oz = OZ.zgemm(A, B)
    assert np.all(oz[3, :] == 0) and np.all(oz[:, 5] == 0)
    ex = A.astype(np.clongdouble) @ B.astype(np.clongdouble)
    assert float(np.linalg.norm(oz - ex) / np.linalg.norm(ex)) < 1e-15
