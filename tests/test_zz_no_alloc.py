"""rg_tdistrib_seed_noalloc: the entry point for callers that cannot allocate
device memory at call time (pool-managed device memory, latency-critical
loops).  It draws the potential into the library's fixed
16 MiB device array instead of allocated scratch; its results must equal the
allocating entry point rg_compute_tdistrib's, on consecutive calls that
reuse the shared array.  Collected last on purpose (file name)."""
import ctypes

import numpy as np
import pytest

import recurgreen_gb300 as rg

pytestmark = pytest.mark.gpu

TN_ABS = 1e-9  # absolute tolerance on transmission eigenvalues, as in the parity tests


def _noalloc(g, seed, torch):
    L = rg.lib()
    out = torch.zeros(g.neigv, dtype=torch.float64, device="cuda")
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()  # an explicit stream: the work is enqueued there and awaited below
    stream.wait_stream(torch.cuda.current_stream())
    rc = L.rg_tdistrib_seed_noalloc(g._h, seed, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.data_ptr()),
                                    ctypes.c_void_p(stream.cuda_stream))
    assert rc == rg.RG_OK, L.rg_last_error().decode()
    stream.synchronize()
    return out.cpu().numpy(), int(st.item())


@pytest.mark.parametrize("kw", [
    dict(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=5.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=64),
    dict(boundtype="dirichlet", nxdiso=300, nxfree=2, wol=32.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=256),
    # above 64 modes: the blocked symmetric kernel's matrices and staging share the array
    dict(boundtype="dirichlet", nxdiso=12, nxfree=1, wol=64.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=512),
    # periodic: the pivoted kernel
    dict(boundtype="periodic", nxdiso=40, nxfree=0, wol=6.3, exfac=1.0, aratio=1.0, dscat=2.0),
])
def test_noalloc_matches_allocating_entry_point(kw):
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    g = rg.Waveguide(**kw)
    seeds = (3, 7)
    ref = np.zeros(max(seeds) * g.neigv)
    for s in seeds:
        g.compute_tdistrib(s, ref)
    for s in seeds:  # two calls in a row on the shared array
        T, status = _noalloc(g, s, torch)
        assert status == rg.RG_OK
        np.testing.assert_allclose(T, ref[(s - 1) * g.neigv: s * g.neigv], rtol=0, atol=TN_ABS)


def test_noalloc_rejects_guides_beyond_capacity():
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    g = rg.Waveguide("dirichlet", nxdiso=10000, nxfree=0, wol=5.25, exfac=1.0, dscat=5.0, ny=256)
    L = rg.lib()
    out = torch.zeros(g.neigv, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.rg_tdistrib_seed_noalloc(g._h, 1, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.data_ptr()), None)
    assert rc == rg.RG_ERR_INVALID_ARG
    assert b"capacity" in L.rg_last_error()
    # seeds below 1 are rejected, as by rg_compute_tdistrib
    small = rg.Waveguide("dirichlet", nxdiso=20, nxfree=0, wol=5.25, exfac=1.0, dscat=5.0, ny=64)
    for bad in (0, -3):
        rc = L.rg_tdistrib_seed_noalloc(small._h, bad, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.data_ptr()),
                                        None)
        assert rc == rg.RG_ERR_INVALID_ARG and b"iseed" in L.rg_last_error()
