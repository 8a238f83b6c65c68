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


def test_balanced_digits_reconstruct_the_fixed_point():
    """The six balanced base-512 digits rebuild the 53-bit fixed point exactly
    and stay within [-256, 256], including all-carry patterns (raw digits of
    256 and 511 everywhere) and the largest and smallest entries of a row."""
    e = np.int64(0)
    # X = |x| 2^(53-e) for x in [0.5, 1) (exponent 0): X spans [2^52, 2^53)
    raw = [(1 << 53) - 1,                      # every raw digit 511 except the top
           sum(256 << (9 * k) for k in range(5)) | (1 << 52),  # every low raw digit exactly 256
           sum(255 << (9 * k) for k in range(5)) | (1 << 52),  # every low raw digit 255: no carry
           1 << 52]
    xs = np.array([X * 2.0 ** -53 for X in raw] + [-0.75, 1e-12, 2.0 ** -60, 0.0])
    ds = OZ.digits(xs, np.full(xs.shape, e))
    X = OZ.fixed53(xs, np.full(xs.shape, e))
    rebuilt = sum(d * (1 << (9 * (OZ.SLICES - 1 - p))) for p, d in enumerate(ds))
    assert np.array_equal(np.abs(rebuilt), X)
    assert np.array_equal(rebuilt < 0, (xs < 0) & (X > 0))
    assert max(int(np.abs(d).max()) for d in ds) <= 256
    # the exactly representable raw values survive the rounding to 53 bits unchanged
    assert [int(v) for v in X[:4]] == raw
