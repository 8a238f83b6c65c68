"""GB300-native recursive Green-function sweep of RecurGreen.

Python mirror of the reference ``waveguide`` module interface
(src/waveguide.f90:13-73) over the C ABI in ``include/recurgreen.h``
(``librecurgreen_gb300.so``, built in-tree by ``recurgreen_gb300.build``).
All computation runs in the CUDA library; this module only moves arguments.
If the library is missing, every entry point raises: there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "librecurgreen_gb300.so")
_LIB = None

RG_OK, RG_ERR_INVALID_ARG, RG_ERR_SINGULAR, RG_ERR_CUDA, RG_ERR_NOMEM, RG_ERR_NOCONV = range(6)
BOUNDTYPES = {"dirichlet": 0, "periodic": 1}

# Every symbol declared in include/recurgreen.h.
EXPORTS = (
    "rg_last_error", "rg_init", "rg_init_copy", "rg_del", "rg_get_nmu", "rg_get_neigv", "rg_get_nx",
    "rg_get_ny", "rg_get_nprop", "rg_get_window", "rg_get_xmesh", "rg_get_parameters", "rg_get_scalars",
    "rg_compute_tdistrib", "rg_compute_refl_trans_v1", "rg_tdistrib_upot", "rg_refl_trans_v1_upot",
    "rg_potential", "rg_tdistrib_batch", "rg_tdistrib_batch_device", "rg_histogram",
    "rg_tdistrib_seed_noalloc", "rg_last_sweep_time", "rg_tdistrib_multi", "rg_sweep_segment",
    "rg_adjoint_grad_rows", "rg_get_modes", "rg_last_batch_info", "rg_refl_trans_v1_batch",
    "rg_tprofile_batch", "rg_compute_tprofile", "rg_compute_itx_profile", "rg_compute_tprofile_group",
    "rg_compute_deposition", "rg_deposition_batch", "rg_compute_wavefunction", "rg_diagonalize_ahca",
    "rg_sweep_states", "rg_compute_refl_trans_v2", "rg_probe_rate",
    "rg_ozaki_zgemm", "rg_zgemm_workspace_bytes", "rg_zgemm_batched",
)
PROFILE_KINDS = {"tprofile": 0, "itx": 1, "group": 2}
KERNELS = {0: "pivoted", 1: "symmetric", 2: "blocked", 3: "blocked_symmetric"}


class RecurGreenError(RuntimeError):
    """A non-zero status from the C ABI (the reference would have stopped)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[status {code}] {msg}")
        self.code = code


class rg_batch_info(C.Structure):
    _fields_ = [("kernel", C.c_int), ("grid", C.c_int), ("cluster", C.c_int), ("rerun", C.c_int)]


class rg_params(C.Structure):
    _fields_ = [("boundtype", C.c_int), ("nxdiso", C.c_int), ("nxfree", C.c_int), ("wol", C.c_double),
                ("exfac", C.c_double), ("aratio", C.c_double), ("dscat", C.c_double), ("dabso", C.c_double),
                ("napera", C.c_double), ("naperb", C.c_double), ("ny", C.c_int)]


def lib() -> C.CDLL:
    """Loads the CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RecurGreenError(RG_ERR_CUDA, f"{LIB_PATH} is missing; run `python -m recurgreen_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp, dp, ip, i64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int64
    L.rg_last_error.restype = C.c_char_p
    L.rg_init.argtypes = [C.POINTER(rg_params), C.POINTER(vp)]
    L.rg_init_copy.argtypes = [vp, C.POINTER(vp)]
    L.rg_del.argtypes = [vp]
    L.rg_del.restype = None
    for f in ("rg_get_nmu", "rg_get_neigv", "rg_get_nx", "rg_get_ny", "rg_get_nprop"):
        getattr(L, f).argtypes = [vp]
    L.rg_get_window.argtypes = [vp] + [C.POINTER(C.c_int)] * 4
    L.rg_get_xmesh.argtypes = [vp, dp, i64]
    L.rg_get_parameters.argtypes = [vp, C.POINTER(rg_params)]
    L.rg_get_scalars.argtypes = [vp, dp, dp, dp]
    L.rg_compute_tdistrib.argtypes = [vp, C.c_int, dp, i64]
    L.rg_compute_refl_trans_v1.argtypes = [vp, C.c_int, vp, vp]
    L.rg_tdistrib_upot.argtypes = [vp, dp, dp, vp]
    L.rg_refl_trans_v1_upot.argtypes = [vp, dp, vp, vp]
    L.rg_potential.argtypes = [vp, C.c_int, dp]
    L.rg_tdistrib_batch.argtypes = [vp, ip, C.c_int, dp, ip]
    L.rg_tdistrib_batch_device.argtypes = [vp, vp, C.c_int, vp, vp, vp]
    L.rg_histogram.argtypes = [dp, i64, dp, C.c_int, dp, dp]
    L.rg_tdistrib_seed_noalloc.argtypes = [vp, C.c_int, vp, vp, vp]
    L.rg_last_sweep_time.argtypes = [vp, C.POINTER(C.c_float)]
    L.rg_tdistrib_multi.argtypes = [C.POINTER(vp), ip, C.c_int, C.POINTER(C.c_int64), dp, i64, ip]
    L.rg_sweep_segment.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp]
    L.rg_adjoint_grad_rows.argtypes = [vp, vp, C.c_int, vp, i64, vp]
    L.rg_get_modes.argtypes = [vp, vp, vp]
    L.rg_last_batch_info.argtypes = [vp, C.POINTER(rg_batch_info)]
    L.rg_refl_trans_v1_batch.argtypes = [vp, ip, C.c_int, vp, vp, ip]
    L.rg_tprofile_batch.argtypes = [vp, ip, C.c_int, C.c_int, C.c_int, dp, dp, dp, ip, dp, ip]
    L.rg_compute_tprofile.argtypes = [vp, C.c_int, C.c_double, C.c_double, dp, i64, C.POINTER(C.c_int)]
    L.rg_compute_itx_profile.argtypes = [vp, C.c_int, C.c_double, C.c_double, dp, i64]
    L.rg_compute_tprofile_group.argtypes = [vp, C.c_int, C.c_int, dp, dp, dp, i64, ip, dp]
    L.rg_compute_deposition.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
    L.rg_deposition_batch.argtypes = [vp, ip, C.c_int, C.c_int, C.c_int, C.c_int, vp, ip]
    L.rg_compute_wavefunction.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, i64]
    L.rg_diagonalize_ahca.argtypes = [vp, C.c_int, C.c_int, dp, vp]
    L.rg_sweep_states.argtypes = [vp, vp, C.c_int, vp, vp, vp, vp, vp]
    L.rg_compute_refl_trans_v2.argtypes = [vp, C.c_int, vp, vp]
    L.rg_probe_rate.argtypes = [C.c_int, C.c_int, dp]
    L.rg_ozaki_zgemm.argtypes = [C.c_int, vp, vp, vp]
    L.rg_zgemm_workspace_bytes.argtypes = [C.c_int, C.c_int]
    L.rg_zgemm_workspace_bytes.restype = C.c_int64
    L.rg_zgemm_batched.argtypes = ([C.c_int, C.c_int, vp, i64, C.c_int, C.c_int, vp, i64, C.c_int, C.c_int, vp,
                                    C.c_double, C.c_double, vp, i64, C.c_int, C.c_double, vp, i64, C.c_int, vp, i64,
                                    vp])
    _LIB = L
    return L


def _check(rc: int) -> None:
    if rc != RG_OK:
        raise RecurGreenError(rc, lib().rg_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Waveguide:
    """The reference ``waveguide_t`` on the GPU.

    ``Waveguide(boundtype, nxdiso, nxfree, wol, exfac, aratio, dscat, dabso,
    napera, naperb)`` mirrors ``init`` (src/waveguide.f90:81-85); ``ny`` is
    the optional transverse grid size (0 keeps the reference's ny = nmu).
    """

    def __init__(self, boundtype: str = "dirichlet", nxdiso: int = 100, nxfree: int = 0, wol: float = 4.3,
                 exfac: float = 1.0, aratio: float = 1.0, dscat: float = 1.0, dabso: float = 0.0,
                 napera: float = 1.0, naperb: float = 1.0, ny: int = 0, _handle=None):
        L = lib()
        if _handle is None:
            p = rg_params(BOUNDTYPES.get(boundtype, -1), nxdiso, nxfree, wol, exfac, aratio, dscat, dabso,
                          napera, naperb, ny)
            h = C.c_void_p()
            _check(L.rg_init(C.byref(p), C.byref(h)))
            _handle = h
        self._h = _handle
        self.nmu = L.rg_get_nmu(self._h)
        self.neigv = L.rg_get_neigv(self._h)
        self.nx = L.rg_get_nx(self._h)
        self.ny = L.rg_get_ny(self._h)
        self.nprop = L.rg_get_nprop(self._h)
        w = [C.c_int() for _ in range(4)]
        _check(L.rg_get_window(self._h, *[C.byref(x) for x in w]))
        self.imin, self.imax, self.jmin, self.jmax = (x.value for x in w)
        p = self.get_parameters()
        self.nxdiso, self.nxfree = p["nxdiso"], p["nxfree"]
        s = [C.c_double() for _ in range(3)]
        _check(L.rg_get_scalars(self._h, *[C.byref(x) for x in s]))
        self.kdx, self.dos, self.stdu = (x.value for x in s)

    # -- construction / destruction (src/waveguide.f90:262-286) --
    def init_copy(self) -> "Waveguide":
        h = C.c_void_p()
        _check(lib().rg_init_copy(self._h, C.byref(h)))
        return Waveguide(_handle=h)

    def delete(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().rg_del(self._h)
            self._h = None

    def __del__(self):
        try:
            self.delete()
        except Exception:
            pass

    # -- getters (src/waveguide.f90:291-350) --
    def get_nmu(self) -> int:
        return self.nmu

    def get_neigv(self) -> int:
        return self.neigv

    def get_nx(self) -> int:
        return self.nx

    def get_xmesh(self) -> np.ndarray:
        x = np.zeros(self.nx, np.float64)
        _check(lib().rg_get_xmesh(self._h, _dp(x), x.size))
        return x

    def get_modes(self):
        """(mumesh, bmat): nmu complex values each (src/waveguide.f90:240-248)."""
        mu = np.zeros(self.nmu, np.complex128)
        b = np.zeros(self.nmu, np.complex128)
        _check(lib().rg_get_modes(self._h, mu.ctypes.data, b.ctypes.data))
        return mu, b

    def get_parameters(self) -> dict:
        p = rg_params()
        _check(lib().rg_get_parameters(self._h, C.byref(p)))
        bt = {v: k for k, v in BOUNDTYPES.items()}[p.boundtype]
        return dict(boundtype=bt, nxdiso=p.nxdiso, nxfree=p.nxfree, wol=p.wol, exfac=p.exfac, aratio=p.aratio,
                    dscat=p.dscat, dabso=p.dabso, napera=p.napera, naperb=p.naperb, ny=p.ny)

    # -- computations --
    def compute_tdistrib(self, iseed: int, tallvals: np.ndarray) -> None:
        """compute_tdistrib (src/waveguide.f90:392-462): fills chunk iseed of tallvals in place."""
        if tallvals.dtype != np.float64 or not tallvals.flags.c_contiguous:
            raise RecurGreenError(RG_ERR_INVALID_ARG, "tallvals must be a contiguous float64 array")
        _check(lib().rg_compute_tdistrib(self._h, int(iseed), _dp(tallvals), tallvals.size))

    def compute_refl_trans_v1(self, iseed: int):
        """compute_refl_trans_v1 (src/waveguide.f90:469-519): (r, t), nmu x nmu complex."""
        t = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        r = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        _check(lib().rg_compute_refl_trans_v1(self._h, int(iseed), r.ctypes.data, t.ctypes.data))
        return r, t

    def refl_trans_v1_batch(self, seeds, want_r: bool = True):
        """compute_refl_trans_v1 for many seeds in batched launches: (r, t),
        each of shape (n, nmu, nmu) (r is None without want_r)."""
        seeds = np.ascontiguousarray(seeds, np.int32)
        n, M = seeds.size, self.nmu
        t = np.zeros((n, M, M), np.complex128)  # each matrix column-major: t[k] holds t^T
        r = np.zeros((n, M, M), np.complex128) if want_r else None
        st = np.zeros(n, np.int32)
        ip = C.POINTER(C.c_int32)
        _check(lib().rg_refl_trans_v1_batch(self._h, seeds.ctypes.data_as(ip), n, r.ctypes.data if want_r else None,
                                             t.ctypes.data, st.ctypes.data_as(ip)))
        return (r.transpose(0, 2, 1) if want_r else None), t.transpose(0, 2, 1)

    def tdistrib_upot(self, upot: np.ndarray, want_t: bool = False):
        """Eigenvalues (and the filtered Fisher-Lee t) for a given potential
        upot (shape (ny, nxdiso) C-order == upot(nxdiso, ny) Fortran order)."""
        upot = np.ascontiguousarray(upot, np.float64)
        if upot.shape != (self.ny, self.nxdiso):
            raise RecurGreenError(RG_ERR_INVALID_ARG, f"upot must have shape {(self.ny, self.nxdiso)}")
        T = np.zeros(self.neigv, np.float64)
        t = np.zeros((self.imax - self.imin + 1, self.jmax - self.jmin + 1), np.complex128, order="F")
        _check(lib().rg_tdistrib_upot(self._h, _dp(upot), _dp(T), t.ctypes.data if want_t else None))
        return (T, t) if want_t else T

    def refl_trans_v1_upot(self, upot: np.ndarray, want_r: bool = False):
        """t (and r) of compute_refl_trans_v1 for a given potential."""
        upot = np.ascontiguousarray(upot, np.float64)
        if upot.shape != (self.ny, self.nxdiso):
            raise RecurGreenError(RG_ERR_INVALID_ARG, f"upot must have shape {(self.ny, self.nxdiso)}")
        t = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        r = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        _check(lib().rg_refl_trans_v1_upot(self._h, _dp(upot), r.ctypes.data if want_r else None, t.ctypes.data))
        return (r, t) if want_r else t

    def compute_refl_trans_v2(self, iseed: int):
        """compute_refl_trans_v2 (src/waveguide.f90:526-553): (r, t) from the
        full block tridiagonal solve."""
        t = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        r = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        _check(lib().rg_compute_refl_trans_v2(self._h, int(iseed), r.ctypes.data, t.ctypes.data))
        return r, t

    def test_green_v1_v2(self, iseed: int):
        """test_green_v1_v2 (src/waveguide.f90:598-623): (||r_v1 - r_v2||,
        ||t_v1 - t_v2||), both expected 0."""
        r1, t1 = self.compute_refl_trans_v1(iseed)
        r2, t2 = self.compute_refl_trans_v2(iseed)
        return float(np.linalg.norm(r1 - r2)), float(np.linalg.norm(t1 - t2))

    def test_unitarity(self, iseed: int, version: int = 1) -> float:
        """test_unitarity (src/waveguide.f90:561-590): ||t^H t + r^H r - 1||
        for the v1 recursion (version 1) or the full solve (version 2)."""
        if version not in (1, 2):
            raise RecurGreenError(RG_ERR_INVALID_ARG, "Unknown recursive Green version (must be 1 or 2), aborting...")
        r, t = self.compute_refl_trans_v1(iseed) if version == 1 else self.compute_refl_trans_v2(iseed)
        d = t.conj().T @ t + r.conj().T @ r - np.eye(self.nmu)
        return float(np.sqrt(np.sum((d * d.conj()).real)))

    def potential(self, iseed: int) -> np.ndarray:
        """The disorder of seed iseed as drawn on the GPU, shape (ny, nxdiso)."""
        u = np.zeros((self.ny, self.nxdiso), np.float64)
        _check(lib().rg_potential(self._h, int(iseed), _dp(u)))
        return u

    def tdistrib_batch(self, seeds, return_status: bool = False):
        """Batched compute_tdistrib: eigenvalues of every seed, shape (n * neigv,)."""
        seeds = np.ascontiguousarray(seeds, np.int32)
        out = np.zeros(seeds.size * self.neigv, np.float64)
        st = np.zeros(seeds.size, np.int32)
        ip = C.POINTER(C.c_int32)
        rc = lib().rg_tdistrib_batch(self._h, seeds.ctypes.data_as(ip), seeds.size, _dp(out), st.ctypes.data_as(ip))
        if return_status:
            return out, st
        _check(rc)
        return out

    # -- full Green function (src/waveguide.f90:636-997) --
    def tprofile_batch(self, seeds, kind: str, a, b, return_status: bool = False):
        """Transmission-eigenstate profiles of many seeds.  kind "tprofile"
        (windows a[w] <= T <= b[w], full t, times 4/nt), "itx" (same windows,
        times 2/(pi wol |b-a|)) or "group" (|T - a[w]| <= b[w], filtered t,
        times 4/nt).  Returns (profiles (n, nprofile, nx), nt (n, nprofile),
        tavg (n,)) [and the status array]."""
        seeds = np.ascontiguousarray(seeds, np.int32)
        a = np.ascontiguousarray(np.atleast_1d(a), np.float64)
        b = np.ascontiguousarray(np.atleast_1d(b), np.float64)
        if a.shape != b.shape:
            raise RecurGreenError(RG_ERR_INVALID_ARG, "window bounds must have the same length")
        n, npf = seeds.size, a.size
        prof = np.zeros((n, npf, self.nx), np.float64)
        nt = np.zeros((n, npf), np.int32)
        tavg = np.zeros(n, np.float64)
        st = np.zeros(n, np.int32)
        ip = C.POINTER(C.c_int32)
        rc = lib().rg_tprofile_batch(self._h, seeds.ctypes.data_as(ip), n, PROFILE_KINDS.get(kind, -1), npf, _dp(a),
                                     _dp(b), _dp(prof), nt.ctypes.data_as(ip), _dp(tavg), st.ctypes.data_as(ip))
        if return_status:
            return prof, nt, tavg, st
        _check(rc)
        return prof, nt, tavg

    def compute_tprofile(self, iseed: int, tmin: float, tmax: float):
        """compute_tprofile (src/waveguide.f90:843-907) -> (tprofile (nx,), nt)."""
        out = np.zeros(self.nx, np.float64)
        nt = C.c_int()
        _check(lib().rg_compute_tprofile(self._h, int(iseed), tmin, tmax, _dp(out), out.size, C.byref(nt)))
        return out, nt.value

    def compute_itx_profile(self, iseed: int, tmin: float, tmax: float) -> np.ndarray:
        """compute_itx_profile (src/waveguide.f90:764-825) -> itx (nx,)."""
        out = np.zeros(self.nx, np.float64)
        _check(lib().rg_compute_itx_profile(self._h, int(iseed), tmin, tmax, _dp(out), out.size))
        return out

    def compute_tprofile_group(self, iseed: int, tm, dt):
        """compute_tprofile_group (src/waveguide.f90:924-997) -> (tprofile
        (nx, nprofile), nt (nprofile,), tavg)."""
        tm = np.ascontiguousarray(tm, np.float64)
        dt = np.ascontiguousarray(dt, np.float64)
        out = np.zeros((tm.size, self.nx), np.float64)  # Fortran (nx, nprofile) memory order
        nt = np.zeros(tm.size, np.int32)
        tavg = C.c_double()
        _check(lib().rg_compute_tprofile_group(self._h, int(iseed), tm.size, _dp(tm), _dp(dt), _dp(out), out.size,
                                               nt.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(tavg)))
        return out.T.copy(), nt, tavg.value

    def compute_deposition(self, iseed: int, fpos: int, ipos: int) -> np.ndarray:
        """compute_deposition (src/waveguide.f90:710-745) -> depmat (nmu, nmu)."""
        d = np.zeros((self.nmu, self.nmu), np.complex128, order="F")
        _check(lib().rg_compute_deposition(self._h, int(iseed), int(fpos), int(ipos), d.ctypes.data))
        return d

    def deposition_batch(self, seeds, fpos: int, ipos: int, col: int = 0, return_status: bool = False):
        """Deposition matrices of many seeds: (n, nmu, nmu), or column col
        (1-based) of each, (n, nmu)."""
        seeds = np.ascontiguousarray(seeds, np.int32)
        n, M = seeds.size, self.nmu
        out = np.zeros((n, M) if col else (n, M, M), np.complex128)
        st = np.zeros(n, np.int32)
        ip = C.POINTER(C.c_int32)
        rc = lib().rg_deposition_batch(self._h, seeds.ctypes.data_as(ip), n, int(fpos), int(ipos), int(col),
                                       out.ctypes.data, st.ctypes.data_as(ip))
        res = out if col else out.transpose(0, 2, 1)
        if return_status:
            return res, st
        _check(rc)
        return res

    def compute_wavefunction(self, iseed: int, ipos: int, imode: int) -> np.ndarray:
        """compute_wavefunction (src/waveguide.f90:636-698) -> wfundata
        (nx*ny, 5): columns x, y, Re psi, Im psi, upot."""
        rows = self.nx * self.ny
        out = np.zeros((5, rows), np.float64)  # column-major (rows, 5)
        _check(lib().rg_compute_wavefunction(self._h, int(iseed), int(ipos), int(imode), _dp(out), rows))
        return out.T.copy()

    def last_batch_info(self) -> dict:
        """Kernel, grid, cluster and pivoted re-runs of the last tdistrib_batch."""
        info = rg_batch_info()
        _check(lib().rg_last_batch_info(self._h, C.byref(info)))
        return {"kernel": KERNELS.get(info.kernel, str(info.kernel)), "grid": info.grid, "cluster": info.cluster,
                "rerun": info.rerun}


def tdistrib_multi(items, return_status: bool = False):
    """Eigenvalues of many (waveguide, seed) items in grouped persistent
    launches.  items: sequence of (Waveguide, seed).  Returns a list of
    per-item eigenvalue arrays (and the status array if asked)."""
    n = len(items)
    if n == 0:
        return ([], np.zeros(0, np.int32)) if return_status else []
    offs = np.zeros(n, np.int64)
    tot = 0
    for k, (w, _) in enumerate(items):
        offs[k] = tot
        tot += w.neigv
    handles = (C.c_void_p * n)(*[w._h for w, _ in items])
    seeds = np.ascontiguousarray([s for _, s in items], np.int32)
    out = np.zeros(tot, np.float64)
    st = np.zeros(n, np.int32)
    ip = C.POINTER(C.c_int32)
    rc = lib().rg_tdistrib_multi(handles, seeds.ctypes.data_as(ip), n, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                 _dp(out), tot, st.ctypes.data_as(ip))
    res = [out[offs[k]: offs[k] + w.neigv].copy() for k, (w, _) in enumerate(items)]
    if return_status:
        return res, st
    _check(rc)
    return res


def diagonalize_ahca(a):
    """diagonalize_ahca (src/base_utils.f90:394-444) on the GPU: (T, U) with
    A^H A = U diag(T) U^H, T descending."""
    a = np.asfortranarray(a, np.complex128)
    m, n = a.shape
    T = np.zeros(n, np.float64)
    U = np.zeros((n, n), np.complex128, order="F")
    _check(lib().rg_diagonalize_ahca(a.ctypes.data, m, n, _dp(T), U.ctypes.data))
    return T, U


def ozaki_zgemm(a, b) -> np.ndarray:
    """C = A B (complex, M x M) through the tensor-core digit path (rg_ozaki_zgemm)."""
    a = np.asfortranarray(a, np.complex128)
    b = np.asfortranarray(b, np.complex128)
    M = a.shape[0]
    assert a.shape == (M, M) and b.shape == (M, M)
    c = np.zeros((M, M), np.complex128, order="F")
    _check(lib().rg_ozaki_zgemm(M, a.ctypes.data, b.ctypes.data, c.ctypes.data))
    return c


def histogram(samples, bins):
    """histogram (src/base_utils.f90:491-516) on the GPU -> (histo, missing)."""
    samples = np.ascontiguousarray(samples, np.float64)
    bins = np.ascontiguousarray(bins, np.float64)
    h = np.zeros(max(bins.size - 1, 0), np.float64)
    miss = C.c_double(0)
    _check(lib().rg_histogram(_dp(samples), samples.size, _dp(bins), bins.size - 1, _dp(h), C.byref(miss)))
    return h, miss.value
