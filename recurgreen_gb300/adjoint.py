"""Differentiable transmission losses: a hand-written adjoint of the sweep.

TransmissionLosses.apply(U, waveguide) returns, per realization, the losses
L1 = Tr(t^H t) and L2 = Tr((t^H t)^2) of the filtered Fisher-Lee matrix t
(src/waveguide.f90:443-445) for potentials U of shape (B, nxdiso, ny)
(float64, CUDA; U[r, ix, iy] is upot(ix, iy) of realization r), and its
backward gives dL/dU for every grid cell.  The reference has no gradients;
this is new functionality behind the same sweep.  Dirichlet guides only.

Two backward methods give the same gradient:

"green" (default when a realization's slice states fit in memory).  With
H the block tridiagonal system matrix and G = H^-1, t = 2i S G(N,1) S on
the filter window (S = diag sqrt(mu)), and dH_nn = -dV_n:
  dL = 2 Re Tr(Gamma^H dt),  dt = -2i S G(N,n) dH_nn G(n,1) S
so the slice-matrix adjoint is Xbar_n^H = K_n = -2i G(n,1) P G(N,n) with
P = S Gamma~^H S (Gamma~ = Gamma embedded in M x M).  A Dirichlet H is
complex symmetric, so G(N,n) = G(n,N)^T, and both columns of G come from one
forward sweep that keeps every slice's (S_n, Z_n) (rg_sweep_states, the
forward loop of solve_block_tridiag, src/base_utils.f90:318-324):
  G(n,1) = Z_n - S_n B G(n+1,1),   G(N,1) = Z_N,
  G(n,N) = -S_n B G(n+1,N),        G(N,N) = S_N
(its backward loop, :327-330, once with the source at slice 1 and once at
slice N).  Per slice: 8 M^3 for each column and 16 M^3 per loss, against
the recursion's reverse mode below, which also recomputes the forward.

"checkpoint" (O(sqrt(Nx)) states).  Forward in segments of K ~ sqrt(Nx)
slices (rg_sweep_segment), keeping only the states at segment ends; reverse
mode through the recursion, with Gamma = dL/dt*:
  Gs1bar_N = -2i conj(S) Gamma conj(S)          (t = 2i S Gs1_N S)
  for n = N-1 .. 0 (states recomputed segment by segment from checkpoints):
    Gssbar_n += -Gs1bar_n (B Gs1_{n-1})^H        (Gs1_n = -Gss_n B Gs1_{n-1})
    Gs1bar_{n-1} = -conj(B) Gss_n^H Gs1bar_n
    Xbar_n = -Gss_n^H Gssbar_n Gss_n^H           (Gss_n = inv(X_n))
    Gssbar_{n-1} = -conj(B) Xbar_n conj(B)       (X_n = A_n - V_n - B Gss_{n-1} B)
  (slice 0: Gs1_0 = Gss_0, so Gssbar_0 += Gs1bar_0).

In both, dL/dU_n = -2 sum Re(Xbar_n[a][c]) chi_a chi_c (rg_adjoint_grad_rows).
The per-slice complex products are batched over realizations and losses
and run on the tensor cores with FP64 accuracy (rg_zgemm_batched, the
digit-split products of the sweep's propagator); the sweeps and the
gradient rows are this library's kernels too.  Only elementwise torch
operations remain around them.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import RecurGreenError, Waveguide, lib

_vp = C.c_void_p


def _ptr(t: torch.Tensor | None):
    return _vp(t.data_ptr()) if t is not None else None


def _check(rc: int) -> None:
    if rc != 0:
        raise RecurGreenError(rc, lib().rg_last_error().decode())


class _Sweeper:
    def __init__(self, wg: Waveguide, U: torch.Tensor, K: int):
        self.wg, self.U, self.B = wg, U, U.shape[0]
        self.M = wg.nmu
        self.nx = wg.nx
        self.K = K
        self.segs = [(b, min(b + K, self.nx)) for b in range(0, self.nx, K)]
        self.stream = torch.cuda.current_stream()
        self.status = torch.zeros(self.B, dtype=torch.int32, device=U.device)
        self.nrow = wg.imax - wg.imin + 1
        self.ncol = wg.jmax - wg.jmin + 1

    def run(self, b, e, state_in, dump=None, out=None, want_t=False):
        last = e == self.nx
        tf = torch.empty(self.B, self.ncol, self.nrow, dtype=torch.complex128, device=self.U.device) if last else None
        teig = torch.empty(self.B, self.wg.neigv, dtype=torch.float64, device=self.U.device) if last else None
        _check(lib().rg_sweep_segment(self.wg._h, _ptr(self.U), self.B, b, e, _ptr(state_in), _ptr(dump), _ptr(out),
                                      _ptr(tf), _ptr(teig), _ptr(self.status), _vp(self.stream.cuda_stream)))
        return tf, teig

    def check_status(self):
        st = self.status.cpu().numpy()
        if np.any(st != 0):
            raise RecurGreenError(int(st[st != 0][0]), "singular slice matrix in the adjoint sweep")


class TransmissionLosses(torch.autograd.Function):
    """(L1, L2) = (Tr t^H t, Tr (t^H t)^2) per realization, with the adjoint backward."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, wg: Waveguide, K: int = 0, method: str = "auto"):
        method = _method(wg, U, method)
        if method == "green":
            U = _check_input(U, wg)
            t = _green_t(wg, U)
            ckpt = torch.empty(0, device=U.device)
            L1, L2 = _losses(t)
        else:
            L1, L2, U, t, ckpt, K = _forward(U, wg, K)
        ctx.save_for_backward(U, t, ckpt)
        ctx.wg, ctx.K, ctx.method = wg, K, method
        return L1, L2

    @staticmethod
    def backward(ctx, g1, g2):
        U, t, ckpt = ctx.saved_tensors
        B, dev = U.shape[0], U.device
        g1 = torch.zeros(B, dtype=torch.float64, device=dev) if g1 is None else g1
        g2 = torch.zeros(B, dtype=torch.float64, device=dev) if g2 is None else g2
        Gamma = g1[:, None, None] * t + g2[:, None, None] * _gamma2(t)
        if ctx.method == "green":
            dU = _green_backward(ctx.wg, U, lambda b0, b1, tc: Gamma[None, b0:b1])
        else:
            dU = _reverse_sweep(ctx.wg, U, ckpt, ctx.K, Gamma[None])
        return dU[0], None, None, None


class _ZGemm:
    """Batched M x M complex products C_k = alpha op(A_k) diag(s) op(B_k) + beta D_k
    on the tensor cores (rg_zgemm_batched), on row-major complex128 tensors
    whose last two dimensions are (M, M).  An operand with fewer items than
    the batch is shared cyclically (item k uses matrix k % len)."""

    def __init__(self, M: int, nmax: int, dev):
        self.M, self.nmax = M, nmax
        nb = int(lib().rg_zgemm_workspace_bytes(M, nmax))
        self.ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        self.stream = _vp(torch.cuda.current_stream().cuda_stream)

    def _op(self, X: torch.Tensor):
        X = X if X.dim() == 3 else X.reshape(-1, self.M, self.M)
        assert X.dtype == torch.complex128 and X.stride(-1) == 1 and X.stride(-2) == self.M
        return _vp(X.data_ptr()), X.stride(0) if X.shape[0] > 1 else 0, X.shape[0]

    def __call__(self, n, A, B, C, opA=0, opB=0, rowscale=None, alpha=1.0, D=None, beta=0.0):
        assert n <= self.nmax
        pa, sa, ma = self._op(A)
        pb, sb, mb = self._op(B)
        pc, sc, _ = self._op(C)
        pd, sd, md = self._op(D) if D is not None else (None, 0, 1)
        alpha = complex(alpha)
        _check(lib().rg_zgemm_batched(self.M, n, pa, sa, ma, opA, pb, sb, mb, opB, _ptr(rowscale), alpha.real,
                                      alpha.imag, pd, sd, md, beta, pc, sc, 0, _vp(self.ws.data_ptr()),
                                      self.ws.numel(), self.stream))
        return C


def _bmm(A: torch.Tensor, B: torch.Tensor, opA: int = 0, opB: int = 0) -> torch.Tensor:
    """op(A) op(B) for batches of square matrices on the tensor cores
    (rg_zgemm_batched); rectangular ones (ragged filter windows) through torch."""
    M = A.shape[-1]
    if A.shape[-2] == M and B.shape[-2:] == (M, M) and M <= 512 and A.is_cuda:
        A, B = A.contiguous(), B.contiguous()
        n = max(A.reshape(-1, M, M).shape[0], B.reshape(-1, M, M).shape[0])
        C = torch.empty(n, M, M, dtype=torch.complex128, device=A.device)
        _ZGemm(M, n, A.device)(n, A, B, C, opA=opA, opB=opB)
        return C.reshape(B.shape if B.dim() >= A.dim() else A.shape)
    f = {0: lambda x: x, 1: lambda x: x.transpose(-1, -2), 2: lambda x: x.conj().transpose(-1, -2)}
    return f[opA](A) @ f[opB](B)


def _check_input(U: torch.Tensor, wg: Waveguide) -> torch.Tensor:
    if wg.get_parameters()["boundtype"] != "dirichlet":
        raise RecurGreenError(1, "the adjoint supports Dirichlet guides only")
    U = U.detach().contiguous()
    if U.dtype != torch.float64 or U.dim() != 3 or U.shape[1:] != (wg.nxdiso, wg.ny) or not U.is_cuda:
        raise RecurGreenError(1, f"U must be a CUDA float64 tensor of shape (B, {wg.nxdiso}, {wg.ny})")
    return U


def _losses(t: torch.Tensor):
    A = _bmm(t, t, opA=2)  # t^H t
    return (t.abs() ** 2).sum((1, 2)), (A.abs() ** 2).sum((1, 2))


def _gamma2(t: torch.Tensor) -> torch.Tensor:
    """dL2/dt* = 2 t (t^H t)."""
    return 2.0 * _bmm(t, _bmm(t, t, opA=2))


def _states_bytes(wg: Waveguide) -> int:
    return 2 * wg.nx * wg.nmu * wg.nmu * 16


def _method(wg: Waveguide, U: torch.Tensor, method: str) -> str:
    """"green" when one realization's states take at most a quarter of the
    free device memory (then realizations run in chunks that fit), else
    "checkpoint"."""
    if method in ("green", "checkpoint"):
        return method
    if method != "auto":
        raise RecurGreenError(1, f"unknown adjoint method '{method}'")
    free, _ = torch.cuda.mem_get_info(U.device)
    return "green" if _states_bytes(wg) <= free // 4 else "checkpoint"


def _chunk(wg: Waveguide, U: torch.Tensor) -> int:
    """Realizations whose states fit in half the free device memory (one
    launch for the differentiation workload, which fills the GPU best)."""
    free, _ = torch.cuda.mem_get_info(U.device)
    return max(1, min(U.shape[0], int((free // 2) // _states_bytes(wg))))


def _states(wg: Waveguide, U: torch.Tensor, keep: bool = True):
    """One forward sweep of the realizations of U, keeping every slice's
    state when asked: (states (n, nx, 2, M, M) or None, t (n, nrow, ncol))."""
    n, M, dev = U.shape[0], wg.nmu, U.device
    nrow, ncol = wg.imax - wg.imin + 1, wg.jmax - wg.jmin + 1
    states = torch.empty(n, wg.nx, 2, M, M, dtype=torch.complex128, device=dev) if keep else None
    tf = torch.empty(n, ncol, nrow, dtype=torch.complex128, device=dev)
    teig = torch.empty(n, wg.neigv, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    _check(lib().rg_sweep_states(wg._h, _ptr(U), n, _ptr(states), _ptr(tf), _ptr(teig), _ptr(st),
                                 _vp(torch.cuda.current_stream().cuda_stream)))
    bad = st.cpu().numpy()
    if np.any(bad != 0):
        raise RecurGreenError(int(bad[bad != 0][0]), "singular slice matrix in the adjoint sweep")
    return states, tf.transpose(1, 2)


def _green_t(wg: Waveguide, U: torch.Tensor) -> torch.Tensor:
    """The filtered t of every realization: one sweep, no states kept."""
    _, t = _states(wg, U, keep=False)
    return t.contiguous()


def _green_backward(wg: Waveguide, U: torch.Tensor, gamma_of):
    """dL/dU (S, B, nxdiso, ny) by the full-Green-function method.  For each
    chunk [b0, b1) of realizations, gamma_of(b0, b1, t_chunk) gives the
    cotangents Gamma (S, b1-b0, nrow, ncol) of the S losses."""
    M, nx, dev = wg.nmu, wg.nx, U.device
    mu, bm = wg.get_modes()
    sq = torch.from_numpy(np.sqrt(mu)).to(dev)
    bvec = torch.from_numpy(bm).to(dev)[:, None]
    r0, c0 = wg.imin - 1, wg.jmin - 1
    nxdiso, ny, nxfree = wg.nxdiso, wg.ny, wg.nxfree
    stream = _vp(torch.cuda.current_stream().cuda_stream)
    c = _chunk(wg, U)
    out = None
    for b0 in range(0, U.shape[0], c):
        b1 = min(b0 + c, U.shape[0])
        states, t = _states(wg, U[b0:b1])
        Gamma = gamma_of(b0, b1, t)
        S = Gamma.shape[0]
        if out is None:
            out = torch.zeros((S,) + tuple(U.shape), dtype=U.dtype, device=dev)
        G = torch.zeros(S, b1 - b0, M, M, dtype=torch.complex128, device=dev)
        G[:, :, r0:r0 + Gamma.shape[2], c0:c0 + Gamma.shape[3]] = Gamma
        P = sq[:, None] * G.conj().transpose(-1, -2) * sq[None, :]  # S Gamma~^H S
        dU = torch.zeros(S, b1 - b0, nxdiso, ny, dtype=U.dtype, device=dev)
        nb = b1 - b0
        zg = _ZGemm(M, S * nb, dev)
        P = P.reshape(S * nb, M, M).contiguous()
        X1 = states[:, nx - 1, 1].clone()  # G(N,1) = Z_N
        XN = states[:, nx - 1, 0].clone()  # G(N,N) = S_N
        Y = torch.empty(S * nb, M, M, dtype=torch.complex128, device=dev)
        K = torch.empty_like(Y)
        bflat = bvec.reshape(M).contiguous()
        for n in reversed(range(nx)):
            if n < nx - 1:
                Sn, Zn = states[:, n, 0], states[:, n, 1]
                zg(nb, Sn, X1, X1, rowscale=bflat, alpha=-1.0, D=Zn, beta=1.0)  # X1 = Z_n - S_n B X1
                zg(nb, Sn, XN, XN, rowscale=bflat, alpha=-1.0)  # XN = -S_n B XN
            idd = n - nxfree
            if 0 <= idd < nxdiso:
                zg(S * nb, X1, P, Y)  # Y = G(n,1) P, G(n,1) shared by the S losses
                zg(S * nb, Y, XN, K, opB=1, alpha=-2j)  # K = -2i Y G(n,N)^T
                _check(lib().rg_adjoint_grad_rows(wg._h, _ptr(K), S * nb, _vp(dU.data_ptr() + 8 * idd * ny),
                                                  nxdiso * ny, stream))
        out[:, b0:b1] = dU
        del states
    return out


def _forward(U: torch.Tensor, wg: Waveguide, K: int):
    """Checkpointed forward sweep: (L1, L2, t, checkpoints, K)."""
    U = _check_input(U, wg)
    K = K or max(1, int(math.ceil(math.sqrt(wg.nx))))
    sw = _Sweeper(wg, U, K)
    M, B = sw.M, sw.B
    ckpt = torch.empty(max(len(sw.segs) - 1, 1), B, 2, M, M, dtype=torch.complex128, device=U.device)
    state = None
    t = None
    for s, (b, e) in enumerate(sw.segs):
        out = ckpt[s] if e < sw.nx else None
        tf, _ = sw.run(b, e, state, out=out)
        if e < sw.nx:
            state = ckpt[s]
        else:
            t = tf.transpose(1, 2).contiguous()  # (B, nrow, ncol)
    sw.check_status()
    L1, L2 = _losses(t)
    return L1, L2, U, t, ckpt, K


def _reverse_sweep(wg: Waveguide, U: torch.Tensor, ckpt: torch.Tensor, K: int, Gamma: torch.Tensor):
    """dL/dU for S cotangent chains at once: Gamma (S, B, nrow, ncol) holds
    dL/dt* of each chain; returns (S, B, nxdiso, ny).  The forward states are
    recomputed once per segment and shared by the chains, whose per-slice
    products run as one batch of S*B matrices."""
    sw = _Sweeper(wg, U, K)
    M, B, dev = sw.M, sw.B, U.device
    S = Gamma.shape[0]
    mu, bm = wg.get_modes()
    sq = torch.from_numpy(np.sqrt(mu)).to(dev)
    bvec = torch.from_numpy(bm).to(dev)
    bc = bvec.conj()
    r0, c0 = wg.imin - 1, wg.jmin - 1
    Gs1bar = torch.zeros(S, B, M, M, dtype=torch.complex128, device=dev)
    Gs1bar[:, :, r0:r0 + sw.nrow, c0:c0 + sw.ncol] = (-2j * sq[r0:r0 + sw.nrow].conj()[:, None] * Gamma
                                                      * sq[c0:c0 + sw.ncol].conj()[None, :])
    Gssbar = torch.zeros_like(Gs1bar)
    dU = torch.zeros((S,) + tuple(U.shape), dtype=U.dtype, device=dev)
    nxdiso, ny, nxfree = wg.nxdiso, wg.ny, wg.nxfree
    zg = _ZGemm(M, S * B, dev)
    Gs1bar_prev = torch.empty_like(Gs1bar)
    Xbar = torch.empty_like(Gs1bar)
    tmp = torch.empty_like(Gs1bar)
    for s in reversed(range(len(sw.segs))):
        b, e = sw.segs[s]
        sin = ckpt[s - 1] if s > 0 else None
        dump = torch.empty(B, e - b, 2, M, M, dtype=torch.complex128, device=dev)
        sw.run(b, e, sin, dump=dump)
        for n in reversed(range(b, e)):
            Gss = dump[:, n - b, 0]  # shared by the S chains
            if n > 0:
                Gs1_prev = dump[:, n - 1 - b, 1] if n - 1 >= b else sin[:, 1]
                bG = (bvec[:, None] * Gs1_prev).contiguous()
                zg(S * B, Gs1bar, bG, Gssbar, opB=2, alpha=-1.0, D=Gssbar, beta=1.0)  # -= Gs1bar (B Gs1)^H
                zg(S * B, Gss, Gs1bar, Gs1bar_prev, opA=2, alpha=-1.0)
                Gs1bar_prev *= bc[:, None]  # -conj(B) Gss^H Gs1bar
            else:
                Gssbar = Gssbar + Gs1bar
            zg(S * B, Gss, Gssbar, tmp, opA=2)
            zg(S * B, tmp, Gss, Xbar, opB=2, alpha=-1.0)  # -Gss^H Gssbar Gss^H
            idd = n - nxfree
            if 0 <= idd < nxdiso:
                # rows of all S*B realizations: dU is (S, B, nxdiso, ny)
                _check(lib().rg_adjoint_grad_rows(wg._h, _ptr(Xbar), S * B, _vp(dU.data_ptr() + 8 * idd * ny),
                                                  nxdiso * ny, _vp(sw.stream.cuda_stream)))
            if n > 0:
                Gssbar = -(bc[:, None] * Xbar * bc[None, :])
                Gs1bar, Gs1bar_prev = Gs1bar_prev, Gs1bar
    sw.check_status()
    return dU


def transmission_losses(U: torch.Tensor, wg: Waveguide, K: int = 0, method: str = "auto"):
    """(Tr t^H t, Tr (t^H t)^2) per realization, differentiable in U.
    method: "green", "checkpoint" or "auto" (green when the states fit)."""
    return TransmissionLosses.apply(U, wg, K, method)


def transmission_losses_and_grads(U: torch.Tensor, wg: Waveguide, K: int = 0, method: str = "auto"):
    """(L1, L2, dL1/dU, dL2/dU) with both gradients from one backward pass:
    the two cotangents (dL1/dt* = t, dL2/dt* = 2 t t^H t) share the states
    and run as one batch.  With the green method the forward sweep that
    keeps the states also gives t, so a realization is swept once.  Same
    values as two torch.autograd.grad calls through transmission_losses."""
    method = _method(wg, U, method)
    if method == "green":
        U = _check_input(U, wg)
        ts = {}

        def gamma_of(b0, b1, t):
            ts[b0] = t
            return torch.stack([t, _gamma2(t)])

        dU = _green_backward(wg, U, gamma_of)
        L1, L2 = _losses(torch.cat([ts[k] for k in sorted(ts)]))
        return L1, L2, dU[0], dU[1]
    L1, L2, Ud, t, ckpt, K = _forward(U, wg, K)
    Gamma = torch.stack([t, _gamma2(t)])
    dU = _reverse_sweep(wg, Ud, ckpt, K, Gamma)
    return L1, L2, dU[0], dU[1]
