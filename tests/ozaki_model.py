"""Exact integer model of the tensor-core complex product (rg_ozaki.cuh).

Test infrastructure: it restates, with numpy integer arithmetic, every step
of the device path -- row/column exponents, 56-bit rounded fixed point,
eight signed 7-bit digits, level sums over chunks of 64 complex k, the
hi/lo int64 fold and the final single rounding -- so the GPU result must
equal it bit for bit.  Level sums are checked to stay below 2^24 (the
exactness condition of FP32 accumulation on the tensor cores).
"""
import numpy as np

SLICES, LMAX, CHUNK = 8, 8, 64
NOEXP = -4096


def fexp(x: np.ndarray) -> np.ndarray:
    """frexp exponent of |x| (|x| < 2^e), NOEXP for zeros and subnormals."""
    bits = np.ascontiguousarray(x, np.float64).view(np.uint64)
    eb = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    return np.where(eb == 0, NOEXP, eb - 1022)


def fixed56(x: np.ndarray, e: np.ndarray) -> np.ndarray:
    """|x| 2^(56-e) rounded to nearest (ties up), as int64 (< 2^56)."""
    bits = np.ascontiguousarray(x, np.float64).view(np.uint64)
    eb = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = ((bits & np.uint64((1 << 52) - 1)) | np.uint64(1 << 52)).astype(np.int64)
    sh = eb - 1019 - e
    out = np.zeros(x.shape, np.int64)
    pos = (eb != 0) & (sh >= 0)
    out[pos] = m[pos] << sh[pos]
    neg = (eb != 0) & (sh < 0) & (-sh <= 54)
    rs = -sh[neg]
    out[neg] = (m[neg] + (np.int64(1) << (rs - 1))) >> rs
    assert out.max(initial=0) < (1 << 56)
    return out


def digits(x: np.ndarray, e: np.ndarray):
    """Signed digits d_p (int64, |d_p| <= 127) of x relative to 2^e (broadcast)."""
    X = fixed56(x, np.broadcast_to(e, x.shape))
    s = np.where(x < 0, -1, 1)
    return [((X >> (49 - 7 * p)) & 127) * s for p in range(SLICES)]


def zgemm(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """C = A B as the tensor-core digit path computes it (complex128)."""
    A = np.asarray(A, np.complex128)
    B = np.asarray(B, np.complex128)
    M = A.shape[0]
    ea = np.maximum(fexp(A.real), fexp(A.imag)).max(axis=1)
    eb = np.maximum(fexp(B.real), fexp(B.imag)).max(axis=0)
    # digit products are summed in float64 BLAS: every term and partial sum is
    # an integer below 2^24, so the sums are exact
    Ar = [d.astype(np.float64) for d in digits(A.real, ea[:, None])]
    Ai = [d.astype(np.float64) for d in digits(A.imag, ea[:, None])]
    Br = [d.astype(np.float64) for d in digits(B.real, eb[None, :])]
    Bi = [d.astype(np.float64) for d in digits(B.imag, eb[None, :])]
    hr = np.zeros((M, M), np.int64)
    hi_ = np.zeros((M, M), np.int64)
    lr = np.zeros((M, M), np.int64)
    li = np.zeros((M, M), np.int64)
    for c in range(0, M, CHUNK):
        ks = slice(c, c + CHUNK)
        for lev in range(LMAX + 1):
            vr = np.zeros((M, M))
            vi = np.zeros((M, M))
            for p in range(max(0, lev - SLICES + 1), min(lev, SLICES - 1) + 1):
                q = lev - p
                vr += Ar[p][:, ks] @ Br[q][ks, :] - Ai[p][:, ks] @ Bi[q][ks, :]
                vi += Ar[p][:, ks] @ Bi[q][ks, :] + Ai[p][:, ks] @ Br[q][ks, :]
            assert np.abs(vr).max() < (1 << 24) and np.abs(vi).max() < (1 << 24)
            vr, vi = vr.astype(np.int64), vi.astype(np.int64)
            if lev <= 3:
                hr += vr << (7 * (3 - lev))
                hi_ += vi << (7 * (3 - lev))
            else:
                lr += vr << (7 * (8 - lev))
                li += vi << (7 * (8 - lev))
    e = ea[:, None] + eb[None, :]
    re = hr.astype(np.float64) * 2.0 ** -35 + lr.astype(np.float64) * 2.0 ** -70
    im = hi_.astype(np.float64) * 2.0 ** -35 + li.astype(np.float64) * 2.0 ** -70
    return np.ldexp(re, e) + 1j * np.ldexp(im, e)
