"""The CPU oracle pinned against RecurGreen's own known answers.

Fixtures come from the reference's tests (tests/golden/make_golden.py reads
src/base_utils.test.f90 and test/*.csv as text).  The physics checks are the
reference's self-tests turned into assertions: flux conservation
(test_unitarity, src/waveguide.f90:561-590, parameters of
src/waveguide.test.f90:62-73) and v1 == v2 (src/waveguide.f90:598-623).
"""
import json
import math
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _kat():
    with open(os.path.join(GOLD, "base_utils_kat.json")) as f:
        return json.load(f)


def _cmat(d):
    a = np.array(d["re_im"], np.float64)
    return (a[:, 0] + 1j * a[:, 1]).reshape(d["shape"])


def test_singular_values_kat():
    g = _kat()["singular_values"]
    s = O.singular_values(_cmat(g["A"]))
    np.testing.assert_allclose(s, g["S_expc"], rtol=0, atol=1e-14)


def test_diagonalize_ahca_kat():
    # eigenvalues of A^H A are the squared singular values (src/base_utils.f90:439)
    g = _kat()
    s = O.singular_values(_cmat(g["singular_values"]["A"]))
    np.testing.assert_allclose(s * s, g["diagonalize_ahca"]["T_expc"], rtol=0, atol=1e-13)


def test_inverse_complex_kat():
    a = _cmat(_kat()["inverse_complex"]["A"])
    ai = O.inverse_complex(a)
    np.testing.assert_allclose(ai @ a, np.eye(4), atol=1e-14)


def test_norm2_complex_kat():
    g = _kat()["norm2_complex"]
    a = _cmat(g["A"])
    assert abs(math.sqrt(float(np.sum((a * a.conj()).real))) - g["expected"]) < 1e-14


def test_histogram_kat():
    g = _kat()["histogram"]
    h, miss = O.histogram(g["samples"], g["bins"])
    assert list(h) == g["histo_expc"] and miss == 0.0
    assert h.sum() + miss == len(g["samples"])


def test_moving_average_kat():
    g = _kat()["moving_average"]
    s = np.array(g["signal"])
    res = [(0.0 + s[i] + s[i + 1]) / 2 for i in range(len(s) - 1)]
    assert res == g["res_expc"]


def test_replot_fixture():
    """plothisto on test/test_data.csv reproduces test/replot_1.distrib.csv."""
    with open(os.path.join(GOLD, "replot_fixture.json")) as f:
        r = json.load(f)
    samples = np.array([np.nan if s is None else s for s in r["samples"]], np.float64)
    bins = O.chebyshev_bins(r["nbins"], r["xmin"], r["xmax"])
    h, miss = O.histogram(samples, bins)
    assert miss == 6.0 and h.sum() == 8.0  # the NaN is neither counted nor missing
    eps10 = np.finfo(np.float64).eps / 10.0
    h = h + eps10
    npts = 0.0
    for v in h:
        npts += v
    rho = h / (npts * np.diff(bins))
    centres = (0.0 + bins[:-1] + bins[1:]) / 2
    ref = np.array(r["rho"])
    np.testing.assert_allclose(centres, ref[:, 0], rtol=1e-15, atol=0)
    np.testing.assert_allclose(rho, ref[:, 1], rtol=1e-14, atol=0)


def test_prepare_distrib_matches_numpy():
    rng = np.random.default_rng(3)
    t = rng.uniform(0, 1, 5000)
    t[:3] = [0.0, 1.0, np.nextafter(1.0, 2.0)]
    rho, miss = O.prepare_distrib(t, 64)
    assert miss == 1.0
    bins = O.chebyshev_bins(64)
    h, _ = O.histogram(t, bins)
    assert abs(np.sum((rho[:, 1]) * np.diff(bins)) - 1.0) < 1e-12
    assert np.allclose(rho[:, 0], (bins[:-1] + bins[1:]) / 2)


def test_rand_normal_moments():
    """random_normal.test.f90:30-47 checks mean, sigma, skewness, kurtosis of 1e6 normals."""
    x = O.rand_normal(1_000_000, 1)
    m = x.mean()
    s = x.std()
    sk = np.mean(((x - m) / s) ** 3)
    ku = np.mean(((x - m) / s) ** 4)
    assert abs(m) < 5e-3 and abs(s - 1) < 5e-3 and abs(sk) < 1e-2 and abs(ku - 3) < 2e-2
    # lag-1 correlation (random_normal.test.f90:66-78)
    assert abs(np.corrcoef(x[:-1], x[1:])[0, 1]) < 5e-3


def test_randi_ansic_wraps():
    v = O.randi_ansic(4, 1)
    s = 1
    exp = []
    for _ in range(4):
        s = (1103515245 * s + 12345) & 0xFFFFFFFF
        exp.append(s - (1 << 32) if s >= 1 << 31 else s)
    assert list(v) == exp


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_unitarity_and_v1_v2(seed):
    """test_unitarity + test_green_v1_v2 with the parameters of src/waveguide.test.f90:62-73."""
    w = O.Waveguide("dirichlet", nxdiso=100, nxfree=20, wol=4.30, exfac=1.2, aratio=1.0, dscat=0.2, dabso=0.0)
    assert (w.nmu, w.nx, w.neigv) == (10, 140, 8)
    u = w.potential(seed)
    r1, t1 = w.refl_trans_v1_upot(u)
    r2, t2 = w.refl_trans_v2_upot(u)
    d = t1.conj().T @ t1 + r1.conj().T @ r1 - np.eye(w.nmu)
    assert np.linalg.norm(d) < 1e-12
    assert np.linalg.norm(t1 - t2) < 1e-12 and np.linalg.norm(r1 - r2) < 1e-12


def test_tdistrib_chunks_and_errors():
    w = O.Waveguide("dirichlet", nxdiso=20, nxfree=0, wol=2.3, exfac=1.0, dscat=1.0)
    tall = np.zeros(3 * w.neigv)
    w.compute_tdistrib(2, tall)
    assert np.all(tall[: w.neigv] == 0) and np.all(tall[2 * w.neigv:] == 0)
    assert np.all(tall[w.neigv: 2 * w.neigv] > 0)
    with pytest.raises(O.OracleError):
        w.compute_tdistrib(4, tall)
    with pytest.raises(O.OracleError):
        w.compute_tdistrib(1, np.zeros(w.neigv + 1))
    with pytest.raises(O.OracleError):
        O.Waveguide("dirichlet", wol=2.5)  # half-integer wol is rejected for Dirichlet


def test_batch_equals_single():
    w = O.Waveguide("dirichlet", nxdiso=30, nxfree=2, wol=3.3, exfac=1.0, dscat=2.0)
    seeds = [5, 1, 9]
    b = w.tdistrib_batch(seeds, nthreads=2)
    for k, s in enumerate(seeds):
        np.testing.assert_array_equal(b[k * w.neigv:(k + 1) * w.neigv], w.tdistrib_upot(w.potential(s)))
