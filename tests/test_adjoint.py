"""The hand-written adjoint behind torch.autograd, both methods (the full
Green function from kept slice states, and the checkpointed reverse sweep),
checked against central finite differences of the CPU oracle (step
1e-6 * sigma_U), with the bar |dL/dU adjoint - FD| <= 1e-6 relative to the
largest sampled gradient, and against each other."""
import numpy as np
import pytest

import oracle as O
import recurgreen_gb300 as rg

pytestmark = pytest.mark.gpu

FD_REL = 1e-6


def _losses_oracle(o, u):
    _, t = o.tdistrib_upot(u, want_t=True)
    A = t.conj().T @ t
    return float(np.sum(np.abs(t) ** 2)), float(np.sum(np.abs(A) ** 2))


def _check(kw, B, K, ncell, seed0, method):
    torch = pytest.importorskip("torch")
    from recurgreen_gb300.adjoint import transmission_losses

    o, g = O.Waveguide(**kw), rg.Waveguide(**kw)
    us = [o.potential(seed0 + r) for r in range(B)]  # (ny, nxdiso) each
    U = torch.tensor(np.stack([u.T for u in us]), dtype=torch.float64, device="cuda", requires_grad=True)
    L1, L2 = transmission_losses(U, g, K, method)
    for r in range(B):  # forward parity: the segmented sweep gives the oracle's losses
        l1, l2 = _losses_oracle(o, us[r])
        assert abs(L1[r].item() - l1) <= 1e-10 * abs(l1) and abs(L2[r].item() - l2) <= 1e-10 * abs(l2)
    rng = np.random.default_rng(seed0)
    h = 1e-6 * o.stdu
    for which, L in (("L1", L1), ("L2", L2)):
        (gU,) = torch.autograd.grad(L.sum(), U, retain_graph=True)
        gU = gU.cpu().numpy()
        for r in range(B):
            cells = [(int(rng.integers(0, o.nxdiso)), int(rng.integers(0, o.ny))) for _ in range(ncell)]
            fd = []
            for ix, iy in cells:
                up, um = us[r].copy(), us[r].copy()
                up[iy, ix] += h
                um[iy, ix] -= h
                k = 0 if which == "L1" else 1
                fd.append((_losses_oracle(o, up)[k] - _losses_oracle(o, um)[k]) / (2 * h))
            fd = np.array(fd)
            adj = np.array([gU[r, ix, iy] for ix, iy in cells])
            scale = np.max(np.abs(fd))
            assert np.max(np.abs(adj - fd)) <= FD_REL * scale, (which, r, np.max(np.abs(adj - fd)) / scale)


@pytest.mark.parametrize("method", ["green", "checkpoint"])
def test_adjoint_small_absorbing(method):
    kw = dict(boundtype="dirichlet", nxdiso=14, nxfree=1, wol=6.25, exfac=1.0, aratio=1.0, dscat=3.0, dabso=0.3,
              ny=24)
    _check(kw, B=2, K=4, ncell=10, seed0=3, method=method)


@pytest.mark.parametrize("method", ["green", "checkpoint"])
def test_adjoint_differentiation_width(method):
    """The differentiation config's modes and grid (M=128, ny=512), a short guide."""
    kw = dict(boundtype="dirichlet", nxdiso=24, nxfree=0, wol=64.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=512)
    _check(kw, B=1, K=5, ncell=6, seed0=11, method=method)


@pytest.mark.parametrize("kw", [
    dict(boundtype="dirichlet", nxdiso=40, nxfree=3, wol=12.25, exfac=1.0, aratio=1.0, dscat=6.0, dabso=0.4, ny=48,
         napera=0.7),
    dict(boundtype="dirichlet", nxdiso=16, nxfree=1, wol=36.25, exfac=1.0, aratio=1.0, dscat=3.0, ny=96),
])
def test_green_and_checkpoint_gradients_agree(kw):
    """The two backward methods on guides below and above 64 modes (a filter
    window, absorption, free slices)."""
    torch = pytest.importorskip("torch")
    from recurgreen_gb300.adjoint import transmission_losses_and_grads

    g = rg.Waveguide(**kw)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(9)
    U = torch.randn(3, g.nxdiso, g.ny, dtype=torch.float64, device="cuda", generator=gen) * g.stdu
    a = transmission_losses_and_grads(U, g, 0, "green")
    b = transmission_losses_and_grads(U, g, 0, "checkpoint")
    for x, y in zip(a[:2], b[:2]):
        assert (torch.abs(x - y) / torch.abs(y)).max().item() <= 1e-10
    for x, y in zip(a[2:], b[2:]):
        assert (torch.linalg.norm(x - y) / torch.linalg.norm(y)).item() <= 1e-9


def test_state_sweep_keeps_the_solve_block_tridiag_pair():
    """rg_sweep_states: the kept (Gss, Gs1) of every slice are the forward
    loop of the oracle's solve_block_tridiag, and t is the tdistrib t."""
    torch = pytest.importorskip("torch")
    from recurgreen_gb300.adjoint import _states

    kw = dict(boundtype="dirichlet", nxdiso=25, nxfree=2, wol=5.25, exfac=1.0, aratio=1.0, dscat=3.0, ny=20)
    g, o = rg.Waveguide(**kw), O.Waveguide(**kw)
    u = o.potential(4)
    U = torch.tensor(u.T[None].copy(), dtype=torch.float64, device="cuda")
    states, t = _states(g, U)
    T1, t1 = g.tdistrib_upot(u, want_t=True)
    assert np.linalg.norm(t[0].cpu().numpy() - t1) / np.linalg.norm(t1) <= 1e-12
    # Z_n, the propagated source, and S_n against the oracle's full solve:
    # G(n,1) = Z_n at the last slice, G(N,N) = S_N
    green = o._green(u, 1)
    np.testing.assert_allclose(states[0, -1, 1].cpu().numpy(), green[-1], rtol=0, atol=1e-12 * np.abs(green[-1]).max())
    gnn = o._green(u, g.nx)[-1]
    np.testing.assert_allclose(states[0, -1, 0].cpu().numpy(), gnn, rtol=0, atol=1e-12 * np.abs(gnn).max())


def test_segmented_forward_matches_one_sweep():
    torch = pytest.importorskip("torch")
    import ctypes

    kw = dict(boundtype="dirichlet", nxdiso=30, nxfree=2, wol=10.25, exfac=1.0, aratio=1.0, dscat=4.0, ny=40)
    g = rg.Waveguide(**kw)
    o = O.Waveguide(**kw)
    u = o.potential(2)
    T1, t1 = g.tdistrib_upot(u, want_t=True)
    U = torch.tensor(u.T[None].copy(), dtype=torch.float64, device="cuda")
    M = g.nmu
    L = rg.lib()
    vp = ctypes.c_void_p
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    s1 = torch.empty(1, 2, M, M, dtype=torch.complex128, device="cuda")
    dump = torch.empty(1, g.nx - 13, 2, M, M, dtype=torch.complex128, device="cuda")
    tf = torch.empty(1, g.jmax - g.jmin + 1, g.imax - g.imin + 1, dtype=torch.complex128, device="cuda")
    te = torch.empty(1, g.neigv, dtype=torch.float64, device="cuda")
    cs = vp(torch.cuda.current_stream().cuda_stream)
    assert L.rg_sweep_segment(g._h, vp(U.data_ptr()), 1, 0, 13, None, None, vp(s1.data_ptr()), None, None,
                              vp(st.data_ptr()), cs) == 0
    assert L.rg_sweep_segment(g._h, vp(U.data_ptr()), 1, 13, g.nx, vp(s1.data_ptr()), vp(dump.data_ptr()), None,
                              vp(tf.data_ptr()), vp(te.data_ptr()), vp(st.data_ptr()), cs) == 0
    torch.cuda.synchronize()
    assert st.item() == 0
    t = tf[0].T.cpu().numpy()
    assert np.linalg.norm(t - t1) / np.linalg.norm(t1) <= 1e-12
    assert np.max(np.abs(te[0].cpu().numpy() - T1)) <= 1e-12
    # the last dumped state is the final slice's: t = 2i S Gs1 S
    mu, _ = g.get_modes()
    sq = np.sqrt(mu)
    gs1 = dump[0, -1, 1].cpu().numpy()
    tt = 2j * sq[:, None] * gs1 * sq[None, :]
    assert np.linalg.norm(tt - t1) / np.linalg.norm(t1) <= 1e-12


@pytest.mark.parametrize("method", ["green", "checkpoint"])
def test_both_gradients_in_one_sweep_match_autograd(method):
    """transmission_losses_and_grads (two cotangent chains in one backward
    pass) equals two torch.autograd.grad calls through transmission_losses."""
    torch = pytest.importorskip("torch")
    from recurgreen_gb300.adjoint import transmission_losses, transmission_losses_and_grads

    kw = dict(boundtype="dirichlet", nxdiso=20, nxfree=1, wol=8.25, exfac=1.0, aratio=1.0, dscat=4.0, dabso=0.2,
              ny=32)
    g = rg.Waveguide(**kw)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    U = torch.randn(3, g.nxdiso, g.ny, dtype=torch.float64, device="cuda", generator=gen) * g.stdu
    U.requires_grad_(True)
    L1, L2 = transmission_losses(U, g, 5, method)
    (a1,) = torch.autograd.grad(L1.sum(), U, retain_graph=True)
    (a2,) = torch.autograd.grad(L2.sum(), U)
    M1, M2, d1, d2 = transmission_losses_and_grads(U.detach(), g, 5, method)
    assert torch.equal(M1, L1.detach()) and torch.equal(M2, L2.detach())
    for ref, got in ((a1, d1), (a2, d2)):
        assert (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item() <= 1e-12
