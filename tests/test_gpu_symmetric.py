"""The symmetric sweep (Dirichlet guides, <= 64 modes) against the pivoted
kernel and the oracle.

With Dirichlet modes every slice matrix is complex symmetric, so the library
eliminates it by a symmetric Gauss-Jordan sweep with diagonal pivots (half
the update work) and hands any realization whose diagonal pivots fall below
RG_SYM_TAU x the largest unswept entry of their row to the pivoted kernel.
RG_SYMMETRIC=0 switches the symmetric kernel off.  The autotuner is off in
these tests so that the kernel under test is the one that runs.

Bars: T_n of the two kernels within 1e-10 absolute (the oracle bar is 1e-9);
t relative Frobenius within 1e-10 of the oracle; a realization the pivoted
kernel re-runs is bit-identical to a pivoted-only run.
"""
import numpy as np
import pytest

import oracle as O
import recurgreen_gb300 as rg

pytestmark = pytest.mark.gpu

TN_ABS = 1e-9
T_REL = 1e-10
KERNEL_ABS = 1e-10

SYM_CASES = {
    "ref_test": dict(boundtype="dirichlet", nxdiso=100, nxfree=20, wol=4.30, exfac=1.2, aratio=1.0, dscat=0.2),
    "small_c1": dict(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=5.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=64),
    "ragged_abs": dict(boundtype="dirichlet", nxdiso=60, nxfree=3, wol=7.3, exfac=1.1, aratio=1.5, dscat=3.0,
                       dabso=0.5, napera=0.6, naperb=1.0, ny=40),
    "m32": dict(boundtype="dirichlet", nxdiso=150, nxfree=0, wol=16.25, exfac=1.0, aratio=1.0, dscat=4.0, ny=128),
    "m64": dict(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=32.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=256),
    "tiny": dict(boundtype="dirichlet", nxdiso=2, nxfree=0, wol=0.7, exfac=1.0, aratio=1.0, dscat=1.0),
}


# Blocked kernel (M > 64): short guides keep the oracle fast.
LARGE_SYM = {
    "m72": dict(boundtype="dirichlet", nxdiso=30, nxfree=2, wol=36.25, exfac=1.0, aratio=1.0, dscat=6.0, ny=96),
    "m100_ragged_abs": dict(boundtype="dirichlet", nxdiso=20, nxfree=0, wol=50.25, exfac=1.0, aratio=1.0,
                            dscat=8.0, dabso=1.0, napera=0.7, naperb=0.9, ny=200),
    "m128": dict(boundtype="dirichlet", nxdiso=16, nxfree=0, wol=64.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=512),
    "m256": dict(boundtype="dirichlet", nxdiso=4, nxfree=0, wol=128.25, exfac=1.0, aratio=1.0, dscat=10.0, ny=1024),
}


@pytest.fixture(autouse=True)
def _no_autotune(monkeypatch):
    monkeypatch.setenv("RG_AUTOTUNE", "0")
    monkeypatch.delenv("RG_SYMMETRIC", raising=False)
    monkeypatch.delenv("RG_SYM_TAU", raising=False)


def batch(kw, seeds, monkeypatch, symmetric=True, tau=None):
    monkeypatch.setenv("RG_SYMMETRIC", "1" if symmetric else "0")
    if tau is None:
        monkeypatch.delenv("RG_SYM_TAU", raising=False)
    else:
        monkeypatch.setenv("RG_SYM_TAU", repr(float(tau)))
    g = rg.Waveguide(**kw)
    out = g.tdistrib_batch(seeds)
    info = g.last_batch_info()
    if g.nmu > 64:
        assert info["kernel"] == ("blocked_symmetric" if symmetric else "blocked")
    else:
        assert info["kernel"] == ("symmetric" if symmetric else "pivoted")
    return out.reshape(len(seeds), g.neigv), info


@pytest.mark.parametrize("name", sorted(SYM_CASES))
def test_symmetric_matches_pivoted_and_oracle(name, monkeypatch):
    kw = SYM_CASES[name]
    seeds = np.arange(1, 33, dtype=np.int32)
    bs, _ = batch(kw, seeds, monkeypatch, symmetric=True)
    bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
    assert np.max(np.abs(bs - bg)) <= KERNEL_ABS, name
    o = O.Waveguide(**kw)
    for k in (0, 5):
        ref = o.tdistrib_upot(o.potential(int(seeds[k])))
        assert np.max(np.abs(bs[k] - ref)) <= TN_ABS, name


@pytest.mark.parametrize("name", ["small_c1", "m64"])
def test_symmetric_t_and_r_against_oracle(name, monkeypatch):
    """Full t (forward sweep) and r (reverse sweep) through the symmetric kernel."""
    monkeypatch.setenv("RG_SYMMETRIC", "1")
    kw = SYM_CASES[name]
    o, g = O.Waveguide(**kw), rg.Waveguide(**kw)
    u = o.potential(3)
    ro, to = o.refl_trans_v1_upot(u)
    r, t = g.refl_trans_v1_upot(u, want_r=True)
    assert np.linalg.norm(t - to) / np.linalg.norm(to) <= T_REL
    assert np.linalg.norm(r - ro) / np.linalg.norm(ro) <= T_REL
    # reciprocity: with Dirichlet modes r is symmetric
    assert np.max(np.abs(r - r.T)) <= 1e-10


def test_every_item_flagged_reruns_bit_identical(monkeypatch):
    """A threshold no pivot can meet sends every realization to the pivoted
    kernel through the device-side flag list; the result is the pivoted-only
    result, bit for bit."""
    kw = SYM_CASES["m32"]
    seeds = np.arange(1, 25, dtype=np.int32)
    bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
    ball, info = batch(kw, seeds, monkeypatch, symmetric=True, tau=1e300)
    assert info["rerun"] == len(seeds)
    np.testing.assert_array_equal(ball, bg)


def test_partial_fallback_each_item_from_one_kernel(monkeypatch):
    """With an intermediate threshold each realization comes either from the
    symmetric kernel (bit-identical to a run that flags nothing) or from the
    pivoted re-run (bit-identical to a pivoted-only run)."""
    kw = SYM_CASES["m32"]
    seeds = np.arange(1, 41, dtype=np.int32)
    bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
    b0, info0 = batch(kw, seeds, monkeypatch, symmetric=True, tau=0.0)
    bmid, info = batch(kw, seeds, monkeypatch, symmetric=True, tau=0.6)
    assert info0["rerun"] == 0
    from_sym = np.all(bmid == b0, axis=1)
    from_piv = np.all(bmid == bg, axis=1)
    assert np.all(from_sym | from_piv)
    assert np.sum(from_piv & ~from_sym) <= info["rerun"] <= np.sum(from_piv)
    assert np.max(np.abs(b0 - bg)) <= KERNEL_ABS


def test_multi_mixed_boundaries(monkeypatch):
    """One multi call whose kernel class holds Dirichlet and periodic guides:
    the symmetric kernel passes the periodic items to the pivoted kernel."""
    monkeypatch.setenv("RG_SYMMETRIC", "1")
    specs = [
        dict(boundtype="dirichlet", nxdiso=50, nxfree=0, wol=5.25, exfac=1.0, dscat=3.0, ny=40),
        dict(boundtype="periodic", nxdiso=40, nxfree=0, wol=4.3, exfac=1.0, dscat=2.0),
        dict(boundtype="dirichlet", nxdiso=30, nxfree=2, wol=6.75, exfac=1.0, dscat=2.0, ny=48, dabso=0.2),
    ]
    gs = [rg.Waveguide(**kw) for kw in specs]
    assert all(g.nmu <= 16 for g in gs)
    items = [(gs[k % 3], 1 + k) for k in range(12)]
    res, st = rg.tdistrib_multi(items, return_status=True)
    assert np.all(st == 0)
    for k in (0, 1, 2):
        o = O.Waveguide(**specs[k])
        g, s = items[k]
        assert np.max(np.abs(res[k] - o.tdistrib_upot(o.potential(s)))) <= TN_ABS
    for (g, s), T in zip(items, res):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(s, one)
        np.testing.assert_array_equal(T, one[(s - 1) * g.neigv:])


@pytest.mark.parametrize("name", sorted(LARGE_SYM))
def test_blocked_symmetric_matches_pivoted_and_oracle(name, monkeypatch):
    kw = LARGE_SYM[name]
    seeds = np.arange(1, 13, dtype=np.int32)
    bs, info = batch(kw, seeds, monkeypatch, symmetric=True)
    bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
    assert info["rerun"] == 0
    assert np.max(np.abs(bs - bg)) <= KERNEL_ABS, name
    o = O.Waveguide(**kw)
    ref = o.tdistrib_upot(o.potential(int(seeds[3])))
    assert np.max(np.abs(bs[3] - ref)) <= TN_ABS, name


def test_blocked_symmetric_t_r_and_single_call(monkeypatch):
    """t and r through the blocked symmetric kernel (r from the reverse
    sweep on a materialised potential), and a single call equals the batch."""
    monkeypatch.setenv("RG_SYMMETRIC", "1")
    kw = LARGE_SYM["m72"]
    o, g = O.Waveguide(**kw), rg.Waveguide(**kw)
    u = o.potential(5)
    ro, to = o.refl_trans_v1_upot(u)
    r, t = g.refl_trans_v1_upot(u, want_r=True)
    assert np.linalg.norm(t - to) / np.linalg.norm(to) <= T_REL
    assert np.linalg.norm(r - ro) / np.linalg.norm(ro) <= T_REL
    d = t.conj().T @ t + r.conj().T @ r - np.eye(g.nmu)
    assert np.linalg.norm(d) < 1e-9  # flux conservation at dabso = 0
    seeds = np.array([3, 8], np.int32)
    b = g.tdistrib_batch(seeds)
    for k, s in enumerate(seeds):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(int(s), one)
        np.testing.assert_array_equal(b[k * g.neigv:(k + 1) * g.neigv], one[(s - 1) * g.neigv:])


def test_blocked_every_item_flagged_reruns_bit_identical(monkeypatch):
    kw = LARGE_SYM["m128"]
    seeds = np.arange(1, 7, dtype=np.int32)
    bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
    ball, info = batch(kw, seeds, monkeypatch, symmetric=True, tau=1e300)
    assert info["rerun"] == len(seeds)
    np.testing.assert_array_equal(ball, bg)


def test_blocked_multi_mixed_boundaries(monkeypatch):
    """The blocked class with Dirichlet and periodic guides of different sizes."""
    monkeypatch.setenv("RG_SYMMETRIC", "1")
    specs = [LARGE_SYM["m72"],
             dict(boundtype="periodic", nxdiso=12, nxfree=0, wol=40.3, exfac=1.0, aratio=1.0, dscat=4.0),
             LARGE_SYM["m100_ragged_abs"]]
    gs = [rg.Waveguide(**kw) for kw in specs]
    items = [(gs[k % 3], 1 + k) for k in range(6)]
    res, st = rg.tdistrib_multi(items, return_status=True)
    assert np.all(st == 0)
    for (g, s), T in zip(items, res):
        one = np.zeros(s * g.neigv)
        g.compute_tdistrib(s, one)
        np.testing.assert_array_equal(T, one[(s - 1) * g.neigv:])
    o = O.Waveguide(**specs[1])
    assert np.max(np.abs(res[1] - o.tdistrib_upot(o.potential(2)))) <= TN_ABS


@pytest.mark.parametrize("wol,ny", [(36.25, 96), (64.25, 512)])
def test_blocked_symmetric_clusters_take_several_items(wol, ny, monkeypatch):
    """Batch sizes that give 8- and 4-CTA clusters with more items than
    co-resident clusters, so each cluster takes a second item: every CTA's
    generator states must be its own (no stale state from the last item)."""
    kw = dict(boundtype="dirichlet", nxdiso=3, nxfree=0, wol=wol, exfac=1.0, aratio=1.0, dscat=5.0, ny=ny)
    for n in (20, 60):
        seeds = np.arange(1, n + 1, dtype=np.int32)
        bs, info = batch(kw, seeds, monkeypatch, symmetric=True)
        bg, _ = batch(kw, seeds, monkeypatch, symmetric=False)
        assert info["cluster"] > 1
        assert np.max(np.abs(bs - bg)) <= KERNEL_ABS, (n, info)
