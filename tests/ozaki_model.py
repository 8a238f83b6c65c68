"""Exact integer model of the tensor-core complex product (rg_ozaki.cuh).

Test infrastructure: it restates, with numpy integer arithmetic, every step
of the device path -- row/column exponents, 53-bit rounded fixed point, six
balanced base-512 digits, level sums over chunks of 16 complex k, the hi/lo
int64 fold and the final single rounding -- so the GPU result must equal it
bit for bit.  Level sums are checked to stay below 2^24 (the exactness
condition of FP32 accumulation on the tensor cores).
"""
import numpy as np

SLICES, BITS, LMAX, HI_LEVELS, CHUNK = 6, 9, 6, 3, 16
NOEXP = -4096


def fexp(x: np.ndarray) -> np.ndarray:
    """frexp exponent of |x| (|x| < 2^e), NOEXP for zeros and subnormals."""
    bits = np.ascontiguousarray(x, np.float64).view(np.uint64)
    eb = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    return np.where(eb == 0, NOEXP, eb - 1022)


def fixed53(x: np.ndarray, e: np.ndarray) -> np.ndarray:
    """|x| 2^(53-e) rounded to nearest (ties up), as int64 (< 2^53)."""
    bits = np.ascontiguousarray(x, np.float64).view(np.uint64)
    eb = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = ((bits & np.uint64((1 << 52) - 1)) | np.uint64(1 << 52)).astype(np.int64)
    rs = e - (eb - 1022)
    out = np.zeros(x.shape, np.int64)
    exact = (eb != 0) & (rs == 0)
    out[exact] = m[exact]
    shr = (eb != 0) & (rs > 0) & (rs <= 54)
    r = rs[shr]
    out[shr] = (m[shr] + (np.int64(1) << (r - 1))) >> r
    assert out.max(initial=0) < (1 << 53)
    return out


def digits(x: np.ndarray, e: np.ndarray):
    """Balanced signed digits d_p (int64, |d_p| <= 256) of x relative to 2^e
    (broadcast): X = sum_p d_p 2^(9(5-p)), built from the least significant
    digit up, a digit of 256 or more becoming digit - 512 with a carry."""
    X = fixed53(x, np.broadcast_to(e, x.shape))
    s = np.where(x < 0, -1, 1)
    d = [None] * SLICES
    carry = np.zeros(X.shape, np.int64)
    for p in range(SLICES - 1, 0, -1):
        t = ((X >> (BITS * (SLICES - 1 - p))) & 511) + carry
        carry = (t >= 256).astype(np.int64)
        d[p] = t - (carry << 9)
    d[0] = (X >> (BITS * (SLICES - 1))) + carry
    assert max(int(np.abs(v).max(initial=0)) for v in d) <= 256
    return [v * s for v in d]


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
            if lev < HI_LEVELS:
                hr += vr << (BITS * (HI_LEVELS - 1 - lev))
                hi_ += vi << (BITS * (HI_LEVELS - 1 - lev))
            else:
                lr += vr << (BITS * (LMAX - lev))
                li += vi << (BITS * (LMAX - lev))
    e = ea[:, None] + eb[None, :]
    re = hr.astype(np.float64) * 2.0 ** -34 + lr.astype(np.float64) * 2.0 ** -70
    im = hi_.astype(np.float64) * 2.0 ** -34 + li.astype(np.float64) * 2.0 ** -70
    return np.ldexp(re, e) + 1j * np.ldexp(im, e)
