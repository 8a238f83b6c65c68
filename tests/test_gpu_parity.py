"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bars (tolerances stated here, from the project's parity contract):
  * t: relative Frobenius error <= 1e-10
  * T_n: absolute error <= 1e-9
  * histogram counts: identical (edges and comparisons are the reference's)
Both sides receive the same potential: the oracle's host-drawn upot is passed
to rg_tdistrib_upot; for seed-driven calls the GPU's own potential is first
checked against the oracle's.
"""
import math

import numpy as np
import pytest

import oracle as O
import recurgreen_gb300 as rg

pytestmark = pytest.mark.gpu

T_REL = 1e-10
TN_ABS = 1e-9


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


CASES = {
    # the reference's own test waveguide (src/waveguide.test.f90:62-73)
    "ref_test": dict(boundtype="dirichlet", nxdiso=100, nxfree=20, wol=4.30, exfac=1.2, aratio=1.0, dscat=0.2),
    # the small plain-method config: kW/pi = 10.5 (M = 10), 200 slices, 64 y points, L/l_s = 5
    "small_c1": dict(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=5.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=64),
    # ragged Fisher-Lee window (napera < naperb) and absorption
    "ragged_abs": dict(boundtype="dirichlet", nxdiso=60, nxfree=3, wol=7.3, exfac=1.1, aratio=1.5, dscat=3.0,
                       dabso=0.5, napera=0.6, naperb=1.0, ny=40),
    "periodic": dict(boundtype="periodic", nxdiso=80, nxfree=0, wol=6.3, exfac=1.0, aratio=1.0, dscat=2.0),
    # M = 32 and M = 64 kernels (the 64-mode kernel at the uniform config's width, shorter guide)
    "m32": dict(boundtype="dirichlet", nxdiso=150, nxfree=0, wol=16.25, exfac=1.0, aratio=1.0, dscat=4.0, ny=128),
    "m64": dict(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=32.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=256),
    # the smallest guide: two slices, one mode
    "tiny": dict(boundtype="dirichlet", nxdiso=2, nxfree=0, wol=0.7, exfac=1.0, aratio=1.0, dscat=1.0),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def pair(request):
    kw = CASES[request.param]
    return request.param, O.Waveguide(**kw), rg.Waveguide(**kw)


def test_init_matches_oracle(pair):
    name, o, g = pair
    assert (g.nmu, g.ny, g.nx, g.neigv, g.nprop) == (o.nmu, o.ny, o.nx, o.neigv, o.nprop)
    assert (g.imin, g.imax, g.jmin, g.jmax) == (o.imin, o.imax, o.jmin, o.jmax)
    assert g.kdx == o.kdx and g.dos == o.dos and g.stdu == o.stdu


def test_potential_matches_oracle(pair):
    name, o, g = pair
    for seed in (1, 17):
        uo, ug = o.potential(seed), g.potential(seed)
        # same stream; log/cos of the device libm may differ by a few ulp
        assert np.max(np.abs(ug - uo)) <= 1e-14 * np.max(np.abs(uo))


def test_tdistrib_upot_parity(pair):
    name, o, g = pair
    for seed in (1, 2, 3):
        u = o.potential(seed)
        To, to = o.tdistrib_upot(u, want_t=True)
        Tg, tg = g.tdistrib_upot(u, want_t=True)
        assert relerr(tg, to) <= T_REL, name
        assert np.max(np.abs(Tg - To)) <= TN_ABS, name
        assert np.all(np.diff(Tg) <= 0)  # descending, like zgesvd


def test_compute_tdistrib_seed_and_chunks(pair):
    name, o, g = pair
    nchunk = 3
    tall = np.zeros(nchunk * g.neigv)
    g.compute_tdistrib(2, tall)
    ref = o.tdistrib_upot(o.potential(2))
    assert np.all(tall[: g.neigv] == 0) and np.all(tall[2 * g.neigv:] == 0)
    assert np.max(np.abs(tall[g.neigv: 2 * g.neigv] - ref)) <= TN_ABS


def test_refl_trans_v1(pair):
    """t and r of compute_refl_trans_v1 (r from the reverse sweep) against the oracle's v1."""
    name, o, g = pair
    u = o.potential(4)
    ro, to = o.refl_trans_v1_upot(u)
    rg_, tg = g.refl_trans_v1_upot(u, want_r=True)
    assert relerr(tg, to) <= T_REL, name
    assert relerr(rg_, ro) <= T_REL, name


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_unitarity_on_gpu(seed):
    """test_unitarity (src/waveguide.f90:561-590) with src/waveguide.test.f90:62-73: flux is
    conserved at dabso = 0, ||t^H t + r^H r - 1|| ~ 0, through the seed-driven C ABI call."""
    g = rg.Waveguide(**CASES["ref_test"])
    assert g.test_unitarity(seed) < 1e-10
    assert g.test_unitarity(seed, version=2) < 1e-10
    # test_green_v1_v2 (src/waveguide.f90:598-623) on src/waveguide.test.f90:95-122's guide
    nr, nt = g.test_green_v1_v2(seed)
    assert nr < 1e-10 and nt < 1e-10
    o = O.Waveguide(**CASES["ref_test"])
    ro, to = o.refl_trans_v1_upot(o.potential(seed))
    r, t = g.compute_refl_trans_v1(seed)
    assert relerr(t, to) <= T_REL and relerr(r, ro) <= T_REL


def test_batch_equals_single_and_oracle():
    kw = CASES["small_c1"]
    g, o = rg.Waveguide(**kw), O.Waveguide(**kw)
    seeds = np.arange(1, 41, dtype=np.int32)
    b = g.tdistrib_batch(seeds)
    ob = o.tdistrib_batch(seeds)
    assert np.max(np.abs(b - ob)) <= TN_ABS
    one = np.zeros(g.neigv * 40)
    g.compute_tdistrib(7, one)
    np.testing.assert_array_equal(one[6 * g.neigv: 7 * g.neigv], b[6 * g.neigv: 7 * g.neigv])


def test_uniform_full_length_two_seeds():
    """The uniform config's full slice matrix size and length (M=64, ny=256, Nx=2000)."""
    kw = dict(boundtype="dirichlet", nxdiso=2000, nxfree=0, wol=32.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=256)
    g, o = rg.Waveguide(**kw), O.Waveguide(**kw)
    for seed in (1, 4096):
        u = o.potential(seed)
        To, to = o.tdistrib_upot(u, want_t=True)
        Tg, tg = g.tdistrib_upot(u, want_t=True)
        assert relerr(tg, to) <= T_REL
        assert np.max(np.abs(Tg - To)) <= TN_ABS
        assert np.all((Tg >= -1e-12) & (Tg <= 1 + 1e-12))  # dabso = 0: 0 <= T <= 1


def test_histogram_matches_oracle():
    rng = np.random.default_rng(11)
    x = rng.uniform(-0.05, 1.05, 200_000)
    bins = O.chebyshev_bins(100)
    x[:6] = [bins[0], bins[-1], bins[37], np.nan, np.nextafter(1.0, 2.0), -0.0]
    hg, mg = rg.histogram(x, bins)
    ho, mo = O.histogram(x, bins)
    np.testing.assert_array_equal(hg, ho)
    assert mg == mo
    assert hg.sum() + mg == x.size - 1  # the NaN is dropped


def test_errors_are_statuses_not_crashes():
    with pytest.raises(rg.RecurGreenError) as e:
        rg.Waveguide("dirichlet", wol=2.5)
    assert e.value.code == rg.RG_ERR_INVALID_ARG
    with pytest.raises(rg.RecurGreenError):
        rg.Waveguide("neumann", wol=2.3)
    g = rg.Waveguide(**CASES["small_c1"])
    with pytest.raises(rg.RecurGreenError) as e:
        g.compute_tdistrib(4, np.zeros(3 * g.neigv))
    assert "chunk" in str(e.value)
    with pytest.raises(rg.RecurGreenError):
        g.compute_tdistrib(1, np.zeros(g.neigv + 1))
    # a NaN in the potential makes every pivot invalid: singular status, context intact
    u = g.potential(1)
    u[:, 0] = np.nan
    with pytest.raises(rg.RecurGreenError) as e:
        g.tdistrib_upot(u)
    assert e.value.code == rg.RG_ERR_SINGULAR
    T = g.tdistrib_upot(g.potential(1))
    assert np.all(np.isfinite(T))


# Many-mode guides go through the blocked large-mode kernel (matrices in
# global memory, potential drawn in-kernel on the seed path).  Short guides
# keep the oracle fast; the slice matrices have the configs' full sizes:
# M=128/ny=512 (differentiation config), M=256/ny=1024 (largest uneven
# width) and M=512/ny=2048 (large sweep config).
LARGE = {
    "m72": dict(boundtype="dirichlet", nxdiso=40, nxfree=2, wol=36.25, exfac=1.0, aratio=1.0, dscat=6.0, ny=96),
    "m81_periodic": dict(boundtype="periodic", nxdiso=30, nxfree=0, wol=40.3, exfac=1.0, aratio=1.0, dscat=4.0),
    "m100_ragged_abs": dict(boundtype="dirichlet", nxdiso=25, nxfree=0, wol=50.25, exfac=1.0, aratio=1.0,
                            dscat=8.0, dabso=1.0, napera=0.7, naperb=0.9, ny=200),
    "m128": dict(boundtype="dirichlet", nxdiso=30, nxfree=0, wol=64.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=512),
    "m256": dict(boundtype="dirichlet", nxdiso=8, nxfree=0, wol=128.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=1024),
    "m512": dict(boundtype="dirichlet", nxdiso=4, nxfree=0, wol=256.25, exfac=1.0, aratio=1.0, dscat=20.0, ny=2048),
}


@pytest.fixture(scope="module", params=sorted(LARGE))
def large_pair(request):
    kw = LARGE[request.param]
    return request.param, O.Waveguide(**kw), rg.Waveguide(**kw)


def test_large_tdistrib_upot_parity(large_pair):
    name, o, g = large_pair
    u = o.potential(5)
    To, to = o.tdistrib_upot(u, want_t=True)
    Tg, tg = g.tdistrib_upot(u, want_t=True)
    assert relerr(tg, to) <= T_REL, name
    assert np.max(np.abs(Tg - To)) <= TN_ABS, name


def test_large_seed_path(large_pair):
    """The in-kernel draw must reproduce the oracle's potential stream."""
    name, o, g = large_pair
    tall = np.zeros(2 * g.neigv)
    g.compute_tdistrib(2, tall)
    ref = o.tdistrib_upot(o.potential(2))
    assert np.all(tall[: g.neigv] == 0)
    assert np.max(np.abs(tall[g.neigv:] - ref)) <= TN_ABS, name


def test_large_refl_trans_v1_t():
    kw = LARGE["m72"]
    o, g = O.Waveguide(**kw), rg.Waveguide(**kw)
    u = o.potential(9)
    ro, to = o.refl_trans_v1_upot(u)
    rg_, tg = g.refl_trans_v1_upot(u, want_r=True)
    assert relerr(tg, to) <= T_REL and relerr(rg_, ro) <= T_REL
    d = tg.conj().T @ tg + rg_.conj().T @ rg_ - np.eye(g.nmu)
    assert np.linalg.norm(d) < 1e-9  # dabso = 0: flux conservation (M=72, full matrices)


def test_large_batch_matches_single():
    kw = dict(LARGE["m72"], nxdiso=12)
    g = rg.Waveguide(**kw)
    seeds = np.array([4, 2, 11], np.int32)
    b = g.tdistrib_batch(seeds)
    for k, s in enumerate(seeds):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(int(s), one)
        np.testing.assert_array_equal(b[k * g.neigv:(k + 1) * g.neigv], one[(s - 1) * g.neigv:])


def test_multi_uneven_matches_single_and_oracle():
    """Uneven sizes in one call (kernel classes 16/32/64/large mixed, absorption on some)."""
    specs = [
        dict(boundtype="dirichlet", nxdiso=50, nxfree=0, wol=5.25, exfac=1.0, dscat=3.0, ny=40),
        dict(boundtype="dirichlet", nxdiso=80, nxfree=0, wol=10.25, exfac=1.0, dscat=6.0, ny=80, dabso=0.3),
        dict(boundtype="dirichlet", nxdiso=60, nxfree=1, wol=20.25, exfac=1.0, dscat=9.0, ny=160),
        dict(boundtype="periodic", nxdiso=40, nxfree=0, wol=12.3, exfac=1.0, dscat=2.0),
        dict(boundtype="dirichlet", nxdiso=20, nxfree=0, wol=36.25, exfac=1.0, dscat=4.0, ny=144, dabso=0.8),
        dict(boundtype="dirichlet", nxdiso=10, nxfree=0, wol=50.25, exfac=1.0, dscat=12.0, ny=200),
    ]
    gs = [rg.Waveguide(**kw) for kw in specs]
    items = [(gs[k % len(gs)], 1 + k) for k in range(18)]
    res, st = rg.tdistrib_multi(items, return_status=True)
    assert np.all(st == 0)
    for (g, s), T in zip(items, res):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(s, one)
        np.testing.assert_array_equal(T, one[(s - 1) * g.neigv:])
    for k in (0, 3, 4, 5):
        o = O.Waveguide(**specs[k])
        g, s = items[k]
        assert np.max(np.abs(res[k] - o.tdistrib_upot(o.potential(s)))) <= TN_ABS


def test_batch_graph_replay_and_autotune(monkeypatch):
    """Repeated batch calls on the same device buffers replay a captured CUDA
    graph; the autotuned kernel choice agrees with the heuristic choice."""
    import ctypes

    import torch

    kw = CASES["m64"]
    g = rg.Waveguide(**kw)
    n = 20
    seeds = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    out = torch.zeros(n * g.neigv, dtype=torch.float64, device="cuda")
    st = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    L = rg.lib()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    vp = ctypes.c_void_p
    res = []
    for _ in range(3):  # capture, then two replays
        out.zero_()
        torch.cuda.synchronize()
        rc = L.rg_tdistrib_batch_device(g._h, vp(seeds.data_ptr()), n, vp(out.data_ptr()), vp(st.data_ptr()),
                                        vp(s.cuda_stream))
        assert rc == 0, L.rg_last_error().decode()
        res.append(out.cpu().numpy().copy())
    assert np.all(st.cpu().numpy() == 0)
    np.testing.assert_array_equal(res[0], res[1])
    np.testing.assert_array_equal(res[0], res[2])
    ms = ctypes.c_float()
    assert L.rg_last_sweep_time(g._h, ctypes.byref(ms)) == 0 and ms.value > 0
    monkeypatch.setenv("RG_AUTOTUNE", "0")
    ref = rg.Waveguide(**kw).tdistrib_batch(np.arange(1, n + 1, dtype=np.int32))
    assert np.max(np.abs(ref - res[0])) <= 1e-12


def test_large_autotuned_cluster_matches():
    """The cluster size only moves work between CTAs: a realization gives the
    same bits whatever cluster the autotuner or the heuristic picks."""
    kw = dict(LARGE["m128"], nxdiso=6)
    g = rg.Waveguide(**kw)
    seeds = np.arange(1, 9, dtype=np.int32)
    b = g.tdistrib_batch(seeds)  # autotuned cluster size
    assert g.last_batch_info()["kernel"] in ("blocked", "blocked_symmetric")
    for k, s in enumerate(seeds[:3]):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(int(s), one)  # single realization: cluster of 8
        np.testing.assert_array_equal(b[k * g.neigv:(k + 1) * g.neigv], one[(s - 1) * g.neigv:])


def test_multi_graph_replays_with_fresh_inputs():
    """rg_tdistrib_multi captures its per-class launches as one CUDA graph and
    replays it while the item composition stays the same: a second call with
    other seeds gives each item's single-call result, and a third call with
    the first seeds gives the first call's bits."""
    specs = [
        dict(boundtype="dirichlet", nxdiso=30, nxfree=0, wol=5.25, exfac=1.0, dscat=3.0, ny=40),
        dict(boundtype="dirichlet", nxdiso=40, nxfree=0, wol=20.25, exfac=1.0, dscat=9.0, ny=160, dabso=0.4),
        dict(boundtype="periodic", nxdiso=30, nxfree=0, wol=12.3, exfac=1.0, dscat=2.0),
        dict(boundtype="dirichlet", nxdiso=8, nxfree=0, wol=50.25, exfac=1.0, dscat=12.0, ny=200),
    ]
    gs = [rg.Waveguide(**kw) for kw in specs]
    first = rg.tdistrib_multi([(gs[k % 4], 1 + k) for k in range(12)])
    second = rg.tdistrib_multi([(gs[k % 4], 101 + k) for k in range(12)])
    third = rg.tdistrib_multi([(gs[k % 4], 1 + k) for k in range(12)])
    for a, b in zip(first, third):
        np.testing.assert_array_equal(a, b)
    for k, T in enumerate(second):
        g, s = gs[k % 4], 101 + k
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(s, one)
        np.testing.assert_array_equal(T, one[(s - 1) * g.neigv:])


@pytest.mark.parametrize("kw", [
    dict(boundtype="dirichlet", nxdiso=12, nxfree=0, wol=50.25, exfac=1.0, dscat=6.0, ny=200),   # blocked, row split
    dict(boundtype="dirichlet", nxdiso=60, nxfree=0, wol=24.25, exfac=1.0, dscat=6.0, ny=96),    # shared memory
])
def test_autotuned_and_untuned_bit_identical(kw, monkeypatch):
    """The autotuner's choices (cluster size and threads per update unit above
    64 modes, CTAs per SM below) change no realization's bits."""
    seeds = np.arange(1, 41, dtype=np.int32)
    tuned = rg.Waveguide(**kw).tdistrib_batch(seeds)
    monkeypatch.setenv("RG_AUTOTUNE", "0")
    plain = rg.Waveguide(**kw).tdistrib_batch(seeds)
    np.testing.assert_array_equal(tuned, plain)
