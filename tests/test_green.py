"""Full Green function: transmission-eigenstate profiles, deposition matrix
and wavefunction (src/waveguide.f90:636-997), and the block tridiagonal solve
and eigen-decomposition they stand on (src/base_utils.f90:296-335,394-444).

CPU tests pin the oracle: solve_block_tridiag against the reference's own
test case (src/base_utils.test.f90:290-371, checked as the reference checks it,
by a dense solve of the assembled system), diagonalize_ahca against its
known answer (src/base_utils.test.f90:419-451), and the full-G solution
against the v1 recursion (the reference's test_green_v1_v2,
src/waveguide.f90:598-623).  GPU tests compare the CUDA path with the
oracle on the potential the GPU draws.

Tolerances: profiles 1e-9 relative (max over slices), deposition 1e-10
relative Frobenius (as t), wavefunction 1e-10 relative to max |psi|;
window counts nt exact.
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


def _carr(d):
    a = np.array(d["re_im"], np.float64)
    z = a[:, 0] + 1j * a[:, 1]
    return z.reshape(d["shape"], order="F" if d["order"] == "fortran" else "C")


# ---------------------------------------------------------------- oracle pins

def test_oracle_block_tridiag_reference_case():
    g = _kat()["solve_block_tridiag"]
    amat, imat = _carr(g["amat"]), _carr(g["imat"])
    b = np.array(g["bdiag"], np.complex128)
    x = O.block_tridiag(amat, b, imat)
    nb, m = amat.shape[0], amat.shape[1]
    h = np.zeros((nb * m, nb * m), np.complex128)
    for i in range(nb):
        h[i * m:(i + 1) * m, i * m:(i + 1) * m] = amat[i]
        if i < nb - 1:
            h[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = np.diag(b)
            h[(i + 1) * m:(i + 2) * m, i * m:(i + 1) * m] = np.diag(b)
    expc = np.linalg.solve(h, imat.reshape(nb * m, -1))
    err = np.linalg.norm(x.reshape(nb * m, -1) - expc) / np.linalg.norm(expc)
    assert err < 1e-14


def test_oracle_diagonalize_ahca_reference_case():
    g = _kat()["diagonalize_ahca"]
    a = _carr(g["A"])
    T, U = O.diagonalize_ahca(a)
    np.testing.assert_allclose(T, g["T_expc"], rtol=0, atol=1e-13)
    assert np.abs(a.conj().T @ a - U @ np.diag(T) @ U.conj().T).max() < 1e-13


@pytest.mark.parametrize("bt,wol", [("dirichlet", 3.3), ("periodic", 2.6)])
def test_oracle_full_green_equals_v1(bt, wol):
    """X_1 -> r and X_nx -> t of the full solve equal the v1 sweep's."""
    w = O.Waveguide(bt, nxdiso=50, nxfree=2, wol=wol, dscat=2.0)
    u = w.potential(5)
    r1, t1 = w.refl_trans_v1_upot(u)
    r2, t2 = w.refl_trans_v2_upot(u)
    dep_t = w.deposition_upot(u, w.nx, 1)
    dep_r = w.deposition_upot(u, 1, 1)
    np.testing.assert_allclose(dep_t, t1, atol=1e-13)
    np.testing.assert_allclose(dep_r - np.eye(w.nmu), r2, atol=1e-13)
    np.testing.assert_allclose(r1, r2, atol=1e-13)


@pytest.mark.parametrize("bt,wol", [("dirichlet", 2.7), ("periodic", 2.6)])
def test_oracle_full_green_equals_dense_inverse(bt, wol):
    """The oracle's solve on the guide's own blocks against numpy's inverse of
    the assembled block tridiagonal matrix (diagonal blocks A_n - V_n,
    off-diagonal blocks B), for sources at the first, an inner and the last
    slice: the general-source solve behind the deposition and wavefunction."""
    o = O.Waveguide(bt, nxdiso=24, nxfree=2, wol=wol, dscat=2.0, dabso=0.2)
    u = o.potential(6)
    M, nx = o.nmu, o.nx
    b = o.tables()["bmat"]
    H = np.zeros((nx * M, nx * M), np.complex128)
    for n in range(nx):
        H[n * M:(n + 1) * M, n * M:(n + 1) * M] = o.amat_upot(u, n)
        if n + 1 < nx:
            H[n * M:(n + 1) * M, (n + 1) * M:(n + 2) * M] = np.diag(b)
            H[(n + 1) * M:(n + 2) * M, n * M:(n + 1) * M] = np.diag(b)
    G = np.linalg.inv(H)
    for ipos in (1, 11, nx):
        g = o._green(u, ipos)
        want = G[:, (ipos - 1) * M:ipos * M].reshape(nx, M, M)
        assert np.max(np.abs(g - want)) <= 1e-11 * np.max(np.abs(want)), ipos


def test_oracle_reciprocity_of_deposition():
    """Dirichlet blocks are complex symmetric, so G(x_f; x_i) = G(x_i; x_f)^T."""
    w = O.Waveguide("dirichlet", nxdiso=40, nxfree=1, wol=2.7, dscat=1.5)
    u = w.potential(2)
    a = w.deposition_upot(u, 30, 7)
    b = w.deposition_upot(u, 7, 30)
    np.testing.assert_allclose(a, b.T, atol=1e-13)


# ---------------------------------------------------------------- GPU parity

def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _pair(bt="dirichlet", **kw):
    import recurgreen_gb300 as rg

    args = dict(nxdiso=80, nxfree=3, wol=4.3, dscat=2.0)
    args.update(kw)
    return rg.Waveguide(bt, **args), O.Waveguide(bt, **args)


def _safe_window(tvals, lo, hi, margin=1e-7):
    """Moves [lo, hi] off any eigenvalue by more than margin, so that the
    selection cannot depend on the last bits of T."""
    for _ in range(50):
        if np.all(np.abs(tvals - lo) > margin) and np.all(np.abs(tvals - hi) > margin):
            return lo, hi
        lo, hi = lo + 0.0137, hi - 0.0071
    raise AssertionError("no safe window")


@pytest.mark.gpu
def test_gpu_diagonalize_ahca_reference_case():
    import recurgreen_gb300 as rg

    g = _kat()["diagonalize_ahca"]
    a = _carr(g["A"])
    T, U = rg.diagonalize_ahca(a)
    np.testing.assert_allclose(T, g["T_expc"], rtol=0, atol=1e-13)
    assert np.abs(a.conj().T @ a - U @ np.diag(T) @ U.conj().T).max() < 1e-13
    assert np.abs(U.conj().T @ U - np.eye(3)).max() < 1e-14
    # against LAPACK's eigenvectors: equal up to a phase
    To, Uo = O.diagonalize_ahca(a)
    ph = np.sum(U.conj() * Uo, axis=0)
    np.testing.assert_allclose(np.abs(ph), 1.0, atol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("bt,kw", [("dirichlet", {}), ("periodic", dict(wol=3.6)),
                                   ("dirichlet", dict(exfac=1.4, dabso=0.5))])
def test_gpu_tprofile_and_itx_match_oracle(bt, kw):
    w, o = _pair(bt, **kw)
    for seed in (1, 6):
        u = w.potential(seed)
        tv = np.linalg.svd(o.refl_trans_v1_upot(u)[1], compute_uv=False) ** 2
        lo, hi = _safe_window(tv, 0.15, 0.95)
        p, nt = w.compute_tprofile(seed, lo, hi)
        po, nto = o.tprofile_upot(u, lo, hi)
        assert nt == nto and nt > 0
        assert _rel(p, po) < 1e-9
        itx = w.compute_itx_profile(seed, lo, hi)
        itxo, _ = o.tprofile_upot(u, lo, hi, itx=True)
        assert _rel(itx, itxo) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("bt,kw", [("dirichlet", dict(napera=0.7)), ("periodic", dict(wol=3.6, napera=0.6))])
def test_gpu_tprofile_group_matches_oracle(bt, kw):
    w, o = _pair(bt, **kw)
    tm0 = np.array([0.1, 0.4, 0.65, 0.9])
    for seed in (2, 3):
        u = w.potential(seed)
        t = o.refl_trans_v1_upot(u)[1][o.imin - 1:o.imax, o.jmin - 1:o.jmax]
        tv = np.linalg.svd(t, compute_uv=False) ** 2
        dt = np.full(4, 0.12)
        for k in range(4):
            lo, hi = _safe_window(tv, tm0[k] - dt[k], tm0[k] + dt[k])
            tm0[k], dt[k] = (lo + hi) / 2, (hi - lo) / 2
            assert np.all(np.abs(np.abs(tv - tm0[k]) - dt[k]) > 1e-9)
        p, nt, tavg = w.compute_tprofile_group(seed, tm0, dt)
        po, nto, tavgo = o.tprofile_group_upot(u, tm0, dt)
        np.testing.assert_array_equal(nt, nto)
        assert abs(tavg - tavgo) < 1e-12
        for k in range(4):
            assert _rel(p[:, k], po[:, k]) < 1e-9 if nt[k] else np.all(p[:, k] == 0)


@pytest.mark.gpu
def test_gpu_tprofile_group_rejects_wider_input_window():
    import recurgreen_gb300 as rg

    w, _ = _pair(napera=1.0, naperb=0.5)
    with pytest.raises(rg.RecurGreenError, match="zgesvd: Invalid number of singular values"):
        w.compute_tprofile_group(1, [0.5], [0.1])


@pytest.mark.gpu
def test_gpu_tprofile_batch_is_the_single_call():
    w, _ = _pair(nxdiso=60)
    seeds = np.arange(1, 9, dtype=np.int32)
    prof, nt, tavg = w.tprofile_batch(seeds, "tprofile", [0.3], [0.97])
    for k in (0, 5):
        p1, n1 = w.compute_tprofile(int(seeds[k]), 0.3, 0.97)
        assert n1 == nt[k, 0]
        np.testing.assert_array_equal(prof[k, 0], p1)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(nxdiso=70), dict(nxdiso=30, nxfree=1, wol=33.3, dscat=0.5)])
def test_gpu_symmetric_and_pivoted_states_agree(monkeypatch, kw):
    """Dirichlet guides keep their slice states from a symmetric sweep (the
    shared-memory kernel up to 64 modes, the blocked one above); with every
    item flagged (RG_SYM_TAU huge) or the symmetric sweep off (RG_SYMMETRIC=0)
    the pivoted blocked kernel keeps them instead."""
    w, o = _pair(**kw)
    seeds = np.arange(1, 7, dtype=np.int32)
    base, nt0, _ = w.tprofile_batch(seeds, "tprofile", [0.2], [0.99])
    dep = w.deposition_batch(seeds, 20, 11)
    for var, val in (("RG_SYM_TAU", "1e300"), ("RG_SYMMETRIC", "0")):
        monkeypatch.setenv(var, val)
        p, nt, _ = w.tprofile_batch(seeds, "tprofile", [0.2], [0.99])
        np.testing.assert_array_equal(nt, nt0)
        assert _rel(p, base) < 1e-10
        d = w.deposition_batch(seeds, 20, 11)
        assert np.linalg.norm(d - dep) / np.linalg.norm(dep) < 1e-10
        monkeypatch.delenv(var)
    u = w.potential(3)
    do = o.deposition_upot(u, 20, 11)
    assert np.linalg.norm(dep[2] - do) / np.linalg.norm(do) < 1e-10


@pytest.mark.gpu
def test_gpu_chunked_batches_equal_one_launch(monkeypatch):
    """Realizations run in chunks bounded by device memory; chunks of 3 give
    the bits of one launch, for the profiles and the deposition."""
    w, _ = _pair("periodic", nxdiso=50, wol=3.6)
    seeds = np.array([5, 1, 9, 2, 7, 3, 8], np.int32)
    p0, nt0, ta0 = w.tprofile_batch(seeds, "group", [0.2, 0.7], [0.2, 0.3])
    d0 = w.deposition_batch(seeds, 30, 4, col=2)
    monkeypatch.setenv("RG_GREEN_CHUNK", "3")
    p1, nt1, ta1 = w.tprofile_batch(seeds, "group", [0.2, 0.7], [0.2, 0.3])
    d1 = w.deposition_batch(seeds, 30, 4, col=2)
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(nt1, nt0)
    np.testing.assert_array_equal(ta1, ta0)
    np.testing.assert_array_equal(d1, d0)


@pytest.mark.gpu
@pytest.mark.parametrize("bt,kw", [("dirichlet", {}), ("periodic", dict(wol=3.6))])
def test_gpu_deposition_matches_oracle(bt, kw):
    w, o = _pair(bt, **kw)
    u = w.potential(4)
    for fpos, ipos in [(w.nx // 2, 1), (w.nx, 1), (1, 1), (10, 40), (w.nx, w.nx), (60, 17)]:
        d = w.compute_deposition(4, fpos, ipos)
        do = o.deposition_upot(u, fpos, ipos)
        assert np.linalg.norm(d - do) / np.linalg.norm(do) < 1e-10, (fpos, ipos)
    seeds = np.array([4, 9, 11], np.int32)
    full = w.deposition_batch(seeds, w.nx // 2 + 1, 1)
    col = w.deposition_batch(seeds, w.nx // 2 + 1, 1, col=3)
    np.testing.assert_array_equal(full[0], w.compute_deposition(4, w.nx // 2 + 1, 1))
    assert np.max(np.abs(col - full[:, :, 2])) <= 1e-12 * np.max(np.abs(full))


@pytest.mark.gpu
def test_gpu_deposition_at_the_ends_is_t_and_r():
    w, _ = _pair(nxdiso=70)
    r, t = w.compute_refl_trans_v1(3)
    np.testing.assert_allclose(w.compute_deposition(3, w.nx, 1), t, atol=1e-10 * np.abs(t).max())
    np.testing.assert_allclose(w.compute_deposition(3, 1, 1) - np.eye(w.nmu), r, atol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("bt,kw,ipos,imode", [("dirichlet", {}, 1, 1), ("dirichlet", {}, 40, 3),
                                              ("periodic", dict(wol=3.6), 20, 1)])
def test_gpu_wavefunction_matches_oracle(bt, kw, ipos, imode):
    w, o = _pair(bt, **kw)
    u = w.potential(7)
    wf = w.compute_wavefunction(7, ipos, imode)
    wo = o.wavefunction_upot(u, ipos, imode)
    assert wf.shape == (w.nx * w.ny, 5)
    np.testing.assert_array_equal(wf[:, [0, 1, 4]], wo[:, [0, 1, 4]])
    psi, psio = wf[:, 2] + 1j * wf[:, 3], wo[:, 2] + 1j * wo[:, 3]
    assert np.max(np.abs(psi - psio)) < 1e-10 * np.max(np.abs(psio))


@pytest.mark.gpu
def test_gpu_full_green_above_64_modes():
    """The blocked sweep with more modes than the shared-memory kernels hold,
    and the back-substitution with several outputs per thread."""
    w, o = _pair(nxdiso=24, nxfree=1, wol=33.3, dscat=0.5)
    assert w.nmu > 64
    u = w.potential(2)
    d = w.compute_deposition(2, 13, 5)
    do = o.deposition_upot(u, 13, 5)
    assert np.linalg.norm(d - do) / np.linalg.norm(do) < 1e-10
    t = o.refl_trans_v1_upot(u)[1]
    tv = np.linalg.svd(t, compute_uv=False) ** 2
    lo, hi = _safe_window(tv, 0.5, 0.99)
    p, nt = w.compute_tprofile(2, lo, hi)
    po, nto = o.tprofile_upot(u, lo, hi)
    assert nt == nto and nt > 0 and _rel(p, po) < 1e-9


@pytest.mark.gpu
def test_gpu_full_green_argument_checks():
    import recurgreen_gb300 as rg

    w, _ = _pair(nxdiso=20)
    cases = [
        (lambda: w.compute_tprofile(1, -0.1, 0.5), "Invalid Tmin, received Tmin=-0.100, expected in [0, 1]"),
        (lambda: w.compute_tprofile(1, 0.1, 1.5), "Invalid Tmax, received Tmax=1.50, expected in [0, 1]"),
        (lambda: w.compute_itx_profile(1, 0.5, 0.5), "Invalid range (Tmin >= Tmax), aborting..."),
        (lambda: w.compute_tprofile_group(1, [1.2], [0.1]), "Invalid transmission value, expected in [0, 1]"),
        (lambda: w.compute_tprofile_group(1, [0.5], [0.6]), "Invalid transmission half-width, expected 0 < dt <= 1/2"),
        (lambda: w.compute_deposition(1, 0, 1), f"Invalid final position index, received fpos=0, expected in 1..{w.nx}"),
        (lambda: w.compute_deposition(1, 1, w.nx + 1),
         f"Invalid initial position index, received ipos={w.nx + 1}, expected in 1..{w.nx}"),
        (lambda: w.compute_wavefunction(1, 1, w.nmu + 1),
         f"Invalid initial mode index, received imode={w.nmu + 1}, expected in 1..{w.nmu}"),
    ]
    for fn, msg in cases:
        with pytest.raises(rg.RecurGreenError) as e:
            fn()
        assert msg in str(e.value), (msg, str(e.value))
        assert e.value.code == rg.RG_ERR_INVALID_ARG
    assert math.isfinite(w.compute_tprofile(1, 0.0, 1.0)[0].sum())


@pytest.mark.gpu
@pytest.mark.parametrize("bt,kw", [("dirichlet", dict(dabso=0.3)), ("periodic", dict(wol=3.6))])
def test_gpu_refl_trans_v2_and_green_v1_v2(bt, kw):
    """compute_refl_trans_v2 (the full solve) equals the oracle's v2 and the GPU's
    v1; test_green_v1_v2 reports norms near zero, as the reference expects."""
    w, o = _pair(bt, **kw)
    r2, t2 = w.compute_refl_trans_v2(5)
    ro, to = o.refl_trans_v2_upot(w.potential(5))
    assert np.linalg.norm(t2 - to) / np.linalg.norm(to) < 1e-10
    assert np.linalg.norm(r2 - ro) / np.linalg.norm(ro) < 1e-10
    nr, nt = w.test_green_v1_v2(5)
    assert nr < 1e-10 * np.linalg.norm(ro) and nt < 1e-10 * np.linalg.norm(to)
