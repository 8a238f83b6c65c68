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


def test_zgemm_batched_ops_sharing_scaling_and_aliasing():
    """rg_zgemm_batched: op(A) diag(s) op(B) with alpha, beta D, operands shared
    cyclically over the batch, row-major storage, C aliasing D -- against numpy
    at FP64-product accuracy."""
    torch = pytest.importorskip("torch")
    from recurgreen_gb300.adjoint import _ZGemm

    M, nb = 48, 6
    rng = np.random.default_rng(5)

    def rnd(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    A, B, D, s = rnd(2, M, M), rnd(nb, M, M), rnd(3, M, M), rnd(M)
    dev = torch.device("cuda")
    tA, tB, tD, ts = (torch.from_numpy(x).to(dev) for x in (A, B, D, s))
    ops = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T}
    zg = _ZGemm(M, nb, dev)
    for opA in (0, 1, 2):
        for opB in (0, 1, 2):
            C = tD[np.arange(nb) % 3].clone()  # C aliases D
            zg(nb, tA, tB, C, opA=opA, opB=opB, rowscale=ts, alpha=0.5 - 2j, D=C, beta=-1.0)
            Cg = C.cpu().numpy()
            for k in range(nb):
                ref = (0.5 - 2j) * (ops[opA](A[k % 2]) @ (s[:, None] * ops[opB](B[k]))) - D[k % 3]
                assert np.linalg.norm(Cg[k] - ref) <= 1e-14 * np.linalg.norm(ref), (opA, opB, k)
