"""Differentiable transmission losses: a hand-written adjoint of the sweep.

TransmissionLosses.apply(U, waveguide) returns, per realization, the losses
L1 = Tr(t^H t) and L2 = Tr((t^H t)^2) of the filtered Fisher-Lee matrix t
(src/waveguide.f90:443-445) for potentials U of shape (B, nxdiso, ny)
(float64, CUDA; U[r, ix, iy] is upot(ix, iy) of realization r), and its
backward gives dL/dU for every grid cell.  The reference has no gradients;
this is new functionality behind the same sweep.

Forward: the sweep runs in segments of K ~ sqrt(Nx) slices on the GPU
(rg_sweep_segment), keeping only the state (Gss, Gs1) at segment ends.

Backward: reverse-mode through the recursion, with Gamma = dL/dt*:
  Gs1bar_N = -2i conj(S) Gamma conj(S)          (t = 2i S Gs1_N S)
  for n = N-1 .. 0 (states recomputed segment by segment from checkpoints):
    Gssbar_n += -Gs1bar_n (B Gs1_{n-1})^H        (Gs1_n = -Gss_n B Gs1_{n-1})
    Gs1bar_{n-1} = -conj(B) Gss_n^H Gs1bar_n
    Xbar_n = -Gss_n^H Gssbar_n Gss_n^H           (Gss_n = inv(X_n))
    dL/dU_n = -2 sum Re(Xbar_n[a][c]) chi_a chi_c (rg_adjoint_grad_rows)
    Gssbar_{n-1} = -conj(B) Xbar_n conj(B)       (X_n = A_n - V_n - B Gss_{n-1} B)
  (slice 0: Gs1_0 = Gss_0, so Gssbar_0 += Gs1bar_0).
The per-slice complex products are batched over realizations (cuBLAS through
torch); the recomputation and the gradient rows are this library's kernels.
Dirichlet guides only.
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
    def forward(ctx, U: torch.Tensor, wg: Waveguide, K: int = 0):
        L1, L2, U, t, ckpt, K = _forward(U, wg, K)
        ctx.save_for_backward(U, t, ckpt)
        ctx.wg, ctx.K = wg, K
        return L1, L2

    @staticmethod
    def backward(ctx, g1, g2):
        U, t, ckpt = ctx.saved_tensors
        B, dev = U.shape[0], U.device
        g1 = torch.zeros(B, dtype=torch.float64, device=dev) if g1 is None else g1
        g2 = torch.zeros(B, dtype=torch.float64, device=dev) if g2 is None else g2
        Gamma = g1[:, None, None] * t + g2[:, None, None] * 2.0 * (t @ (t.conj().transpose(1, 2) @ t))
        dU = _reverse_sweep(ctx.wg, U, ckpt, ctx.K, Gamma[None])
        return dU[0], None, None


def _forward(U: torch.Tensor, wg: Waveguide, K: int):
    """Checkpointed forward sweep: (L1, L2, t, checkpoints, K)."""
    if wg.get_parameters()["boundtype"] != "dirichlet":
        raise RecurGreenError(1, "the adjoint supports Dirichlet guides only")
    U = U.detach().contiguous()
    if U.dtype != torch.float64 or U.dim() != 3 or U.shape[1:] != (wg.nxdiso, wg.ny) or not U.is_cuda:
        raise RecurGreenError(1, f"U must be a CUDA float64 tensor of shape (B, {wg.nxdiso}, {wg.ny})")
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
    A = t.conj().transpose(1, 2) @ t
    L1 = (t.abs() ** 2).sum((1, 2))
    L2 = (A.abs() ** 2).sum((1, 2))
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
    for s in reversed(range(len(sw.segs))):
        b, e = sw.segs[s]
        sin = ckpt[s - 1] if s > 0 else None
        dump = torch.empty(B, e - b, 2, M, M, dtype=torch.complex128, device=dev)
        sw.run(b, e, sin, dump=dump)
        for n in reversed(range(b, e)):
            Gss = dump[:, n - b, 0]
            GssH = Gss.conj().transpose(1, 2)
            if n > 0:
                Gs1_prev = dump[:, n - 1 - b, 1] if n - 1 >= b else sin[:, 1]
                Gssbar = Gssbar - Gs1bar @ (bvec[:, None] * Gs1_prev).conj().transpose(1, 2)
                Gs1bar_prev = -(bc[:, None] * (GssH @ Gs1bar))
            else:
                Gssbar = Gssbar + Gs1bar
            Xbar = (-(GssH @ Gssbar) @ GssH).contiguous()
            idd = n - nxfree
            if 0 <= idd < nxdiso:
                # rows of all S*B realizations: dU is (S, B, nxdiso, ny)
                _check(lib().rg_adjoint_grad_rows(wg._h, _ptr(Xbar), S * B, _vp(dU.data_ptr() + 8 * idd * ny),
                                                  nxdiso * ny, _vp(sw.stream.cuda_stream)))
            if n > 0:
                Gssbar = -(bc[:, None] * Xbar * bc[None, :])
                Gs1bar = Gs1bar_prev
    sw.check_status()
    return dU


def transmission_losses(U: torch.Tensor, wg: Waveguide, K: int = 0):
    """(Tr t^H t, Tr (t^H t)^2) per realization, differentiable in U."""
    return TransmissionLosses.apply(U, wg, K)


def transmission_losses_and_grads(U: torch.Tensor, wg: Waveguide, K: int = 0):
    """(L1, L2, dL1/dU, dL2/dU) with both gradients from one reverse sweep:
    the two cotangent chains (dL1/dt* = t, dL2/dt* = 2 t t^H t) share the
    recomputed forward states and run as one batch.  Same values as two
    torch.autograd.grad calls through transmission_losses."""
    L1, L2, Ud, t, ckpt, K = _forward(U, wg, K)
    Gamma = torch.stack([t, 2.0 * (t @ (t.conj().transpose(1, 2) @ t))])
    dU = _reverse_sweep(wg, Ud, ckpt, K, Gamma)
    return L1, L2, dU[0], dU[1]
