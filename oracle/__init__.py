"""CPU oracle for the recursive Green-function sweep (test infrastructure only).

This package wraps ``rg_oracle.c`` -- a plain-C restatement of the reference
Fortran algorithm (``src/waveguide.f90``, ``src/base_utils.f90``,
``src/random_normal.f90``, ``src/main.f90`` of RecurGreen) that calls the same
LAPACK routines (zgetrf/zgetri/zgesvd, zgemm for ``matmul``) through the LP64
OpenBLAS bundled with scipy.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may use it, and only as the checker; the
product library never imports it.

Potential-level parity (the gfortran xoshiro256** restatement) is unpinned:
no gfortran >= 9 runtime exists in the build image.  Parity tests therefore
feed the same potential to the oracle and to the GPU path.
"""
from __future__ import annotations

import ctypes as C
import glob
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DIRICHLET, PERIODIC = 0, 1


def build(force: bool = False) -> str:
    """Compile liboracle.so next to this file (gcc, no GPU needed)."""
    so = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "rg_oracle.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return so


def _find_openblas() -> tuple[str, str]:
    import scipy

    d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    cands = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    cands = [c for c in cands if "openblas64" not in os.path.basename(c)]
    if not cands:
        raise RuntimeError("no LP64 scipy OpenBLAS found in " + d)
    return os.path.abspath(cands[0]), "scipy_"


def lib() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    L = C.CDLL(build())
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_void_p
    L.orc_last_error.restype = C.c_char_p
    L.orc_load_lapack.argtypes = [C.c_char_p, C.c_char_p]
    L.orc_init.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 7 + [C.c_int, C.POINTER(vp)]
    L.orc_free.argtypes = [vp]
    L.orc_get_int.argtypes = [vp, C.c_char_p]
    L.orc_get_real.argtypes = [vp, C.c_char_p]
    L.orc_get_real.restype = C.c_double
    L.orc_get_tables.argtypes = [vp, vp, vp, vp, vp]
    L.orc_potential.argtypes = [vp, C.c_int32, dp]
    L.orc_rand_normal.argtypes = [dp, C.c_int64, C.c_int32]
    L.orc_randi_ansic.argtypes = [ip, C.c_int, C.c_int32]
    L.orc_inverse_complex.argtypes = [vp, C.c_int]
    L.orc_singular_values.argtypes = [vp, C.c_int, C.c_int, dp]
    L.orc_tdistrib_upot.argtypes = [vp, dp, dp, vp]
    L.orc_refl_trans_v1_upot.argtypes = [vp, dp, vp, vp]
    L.orc_refl_trans_v2_upot.argtypes = [vp, dp, vp, vp]
    L.orc_compute_tdistrib.argtypes = [vp, C.c_int32, dp, C.c_int64]
    L.orc_tdistrib_batch.argtypes = [vp, ip, C.c_int, dp, C.c_int]
    L.orc_histogram.argtypes = [dp, C.c_int64, dp, C.c_int, dp, dp]
    L.orc_prepare_distrib.argtypes = [dp, C.c_int64, C.c_int, dp, dp]
    L.orc_diagonalize_ahca.argtypes = [vp, C.c_int, C.c_int, dp, vp]
    L.orc_get_modal.argtypes = [vp, vp]
    L.orc_get_meshes.argtypes = [vp, dp, dp]
    L.orc_solve_block_tridiag.argtypes = [vp, dp, vp, C.c_int, vp]
    L.orc_block_tridiag.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp]
    L.orc_amat.argtypes = [vp, dp, C.c_int, vp]
    path, prefix = _find_openblas()
    rc = L.orc_load_lapack(path.encode(), prefix.encode())
    if rc:
        raise RuntimeError(L.orc_last_error().decode())
    _LIB = L
    return L


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"oracle status {code}: {msg}")
        self.code = code


def _check(rc: int) -> None:
    if rc:
        raise OracleError(rc, lib().orc_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Waveguide:
    """Oracle counterpart of the reference ``waveguide_t`` (src/waveguide.f90:13-73)."""

    def __init__(self, boundtype="dirichlet", nxdiso=100, nxfree=0, wol=4.3, exfac=1.0,
                 aratio=1.0, dscat=1.0, dabso=0.0, napera=1.0, naperb=1.0, ny=0):
        L = lib()
        bt = {"dirichlet": DIRICHLET, "periodic": PERIODIC}.get(boundtype, -1)
        h = C.c_void_p()
        _check(L.orc_init(bt, nxdiso, nxfree, wol, exfac, aratio, dscat, dabso, napera, naperb,
                          ny, C.byref(h)))
        self._h = h
        for k in ("nmu", "ny", "nx", "neigv", "nprop", "imin", "imax", "jmin", "jmax"):
            setattr(self, k, L.orc_get_int(h, k.encode()))
        for k in ("kdx", "dos", "stdu"):
            setattr(self, k, L.orc_get_real(h, k.encode()))
        self.nxdiso, self.nxfree = nxdiso, nxfree
        self.wol, self.boundtype = wol, boundtype

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _LIB is not None:
            _LIB.orc_free(h)
            self._h = None

    def tables(self):
        n = self.nmu
        mu, b, ae, ab = (np.zeros(n, np.complex128) for _ in range(4))
        lib().orc_get_tables(self._h, mu.ctypes.data, b.ctypes.data, ae.ctypes.data, ab.ctypes.data)
        return {"mumesh": mu, "bmat": b, "adiag_edge": ae, "adiag_bulk": ab}

    def potential(self, iseed: int) -> np.ndarray:
        """upot(nxdiso, ny) as a C-ordered (ny, nxdiso) array (x fastest)."""
        u = np.zeros((self.ny, self.nxdiso), np.float64)
        lib().orc_potential(self._h, iseed, _dp(u))
        return u

    def tdistrib_upot(self, upot: np.ndarray, want_t: bool = False):
        upot = np.ascontiguousarray(upot, np.float64)
        assert upot.shape == (self.ny, self.nxdiso)
        T = np.zeros(self.neigv, np.float64)
        mr, mc = self.imax - self.imin + 1, self.jmax - self.jmin + 1
        t = np.zeros((mc, mr), np.complex128)  # column-major (mr x mc) buffer
        _check(lib().orc_tdistrib_upot(self._h, _dp(upot), _dp(T), t.ctypes.data if want_t else None))
        return (T, t.T.copy()) if want_t else T

    def refl_trans_v1_upot(self, upot: np.ndarray):
        upot = np.ascontiguousarray(upot, np.float64)
        n = self.nmu
        r = np.zeros((n, n), np.complex128)
        t = np.zeros((n, n), np.complex128)
        _check(lib().orc_refl_trans_v1_upot(self._h, _dp(upot), r.ctypes.data, t.ctypes.data))
        return r.T.copy(), t.T.copy()

    def refl_trans_v2_upot(self, upot: np.ndarray):
        upot = np.ascontiguousarray(upot, np.float64)
        n = self.nmu
        r = np.zeros((n, n), np.complex128)
        t = np.zeros((n, n), np.complex128)
        _check(lib().orc_refl_trans_v2_upot(self._h, _dp(upot), r.ctypes.data, t.ctypes.data))
        return r.T.copy(), t.T.copy()

    # -- full Green function (src/waveguide.f90:636-997) --
    def modal(self) -> np.ndarray:
        m = np.zeros((self.nmu, self.ny), np.complex128)  # column-major (ny, nmu)
        lib().orc_get_modal(self._h, m.ctypes.data)
        return m.T.copy()

    def meshes(self):
        x = np.zeros(self.nx, np.float64)
        y = np.zeros(self.ny, np.float64)
        lib().orc_get_meshes(self._h, _dp(x), _dp(y))
        return x, y

    def amat_upot(self, upot: np.ndarray, ix: int) -> np.ndarray:
        """The diagonal block of slice ix (0-based), set_hamiltonian_waveguide
        (src/waveguide.f90:349-384)."""
        upot = np.ascontiguousarray(upot, np.float64)
        a = np.zeros((self.nmu, self.nmu), np.complex128)  # column-major buffer
        lib().orc_amat(self._h, _dp(upot), ix, a.ctypes.data)
        return a.T.copy()

    def solve_block_tridiag_upot(self, upot: np.ndarray, ind: np.ndarray) -> np.ndarray:
        """solve_block_tridiag (src/base_utils.f90:296-335) on this guide's
        blocks: ind and the result have shape (nx, nmu, k)."""
        upot = np.ascontiguousarray(upot, np.float64)
        nx, M, k = ind.shape
        assert nx == self.nx and M == self.nmu
        buf = np.ascontiguousarray(ind.transpose(0, 2, 1), np.complex128)  # column-major blocks
        x = np.zeros_like(buf)
        _check(lib().orc_solve_block_tridiag(self._h, _dp(upot), buf.ctypes.data, k, x.ctypes.data))
        return x.transpose(0, 2, 1).copy()

    def _green(self, upot, ipos: int, cols=None) -> np.ndarray:
        """G(x_n; x_ipos) for all n: the identity source at block ipos (or
        the unit vectors of the 0-based mode indices `cols`)."""
        M = self.nmu
        k = M if cols is None else len(cols)
        ind = np.zeros((self.nx, M, k), np.complex128)
        if cols is None:
            ind[ipos - 1] = np.eye(M)
        else:
            for q, c in enumerate(cols):
                ind[ipos - 1, c, q] = 1.0
        return self.solve_block_tridiag_upot(upot, ind)

    def _sqmu(self) -> np.ndarray:
        return np.sqrt(self.tables()["mumesh"].real).astype(np.complex128)

    def tprofile_upot(self, upot, tmin: float, tmax: float, itx: bool = False):
        """compute_tprofile (src/waveguide.f90:843-907), or with itx
        compute_itx_profile (src/waveguide.f90:764-825): (profile, nt)."""
        green = self._green(upot, 1)
        sq = self._sqmu()
        tmat = 2.0j * (sq[:, None] * green[self.nx - 1] * sq[None, :])
        tvals, U = diagonalize_ahca(tmat)
        prof = np.zeros(self.nx, np.float64)
        nt = 0
        for iv in range(self.nmu):
            if tmin <= tvals[iv] and tvals[iv] <= tmax:
                for ix in range(self.nx):
                    vec = green[ix] @ (sq * U[:, iv])
                    prof[ix] = prof[ix] + np.sum((vec * vec.conj()).real)
                nt += 1
        if itx:
            prof = prof * 2.0 / (math.pi * self.wol * abs(tmax - tmin))
        elif nt != 0:
            prof = prof * (4.0 / nt)
        return prof, nt

    def tprofile_group_upot(self, upot, tm, dt):
        """compute_tprofile_group (src/waveguide.f90:924-997): (tprofile
        (nx, nprofile), nt (nprofile,), tavg)."""
        green = self._green(upot, 1)
        sq = self._sqmu()
        i0, i1, j0, j1 = self.imin - 1, self.imax, self.jmin - 1, self.jmax
        tmat = 2.0j * (sq[i0:i1, None] * green[self.nx - 1][i0:i1, j0:j1] * sq[None, j0:j1])
        if self.neigv != j1 - j0:
            raise OracleError(1, "zgesvd: Invalid number of singular values")
        tvals, U = diagonalize_ahca(tmat)
        tavg = np.sum(tvals) / self.neigv
        npf = len(tm)
        prof = np.zeros((self.nx, npf), np.float64)
        nt = np.zeros(npf, np.int32)
        for ip in range(npf):
            for iv in range(self.neigv):
                if abs(tvals[iv] - tm[ip]) <= dt[ip]:
                    for ix in range(self.nx):
                        vec = green[ix][:, j0:j1] @ (sq[j0:j1] * U[:, iv])
                        prof[ix, ip] = prof[ix, ip] + np.sum((vec * vec.conj()).real)
                    nt[ip] += 1
            if nt[ip] != 0:
                prof[:, ip] = prof[:, ip] * (4.0 / nt[ip])
        return prof, nt, tavg

    def deposition_upot(self, upot, fpos: int, ipos: int) -> np.ndarray:
        """compute_deposition (src/waveguide.f90:710-745): depmat (nmu, nmu)."""
        green = self._green(upot, ipos)
        sq = self._sqmu()
        return 2.0j * (sq[:, None] * green[fpos - 1] * sq[None, :])

    def wavefunction_upot(self, upot, ipos: int, imode: int) -> np.ndarray:
        """compute_wavefunction (src/waveguide.f90:636-698): (nx*ny, 5)."""
        M = self.nmu
        imu = (imode + M // 2 - 1) % M + 1 if self.boundtype == "periodic" else imode
        green = self._green(upot, ipos, cols=[imu - 1])
        modal = self.modal()
        x, y = self.meshes()
        out = np.zeros((self.nx * self.ny, 5), np.float64)
        for ix in range(self.nx):
            psi = modal @ green[ix, :, 0]
            rows = slice(ix * self.ny, (ix + 1) * self.ny)
            out[rows, 0] = x[ix]
            out[rows, 1] = y
            out[rows, 2] = psi.real
            out[rows, 3] = psi.imag
        u = np.asarray(upot)
        for ix in range(self.nxdiso):
            out[(ix + self.nxfree) * self.ny:(ix + self.nxfree + 1) * self.ny, 4] = u[:, ix]
        return out

    def compute_tdistrib(self, iseed: int, tallvals: np.ndarray) -> None:
        assert tallvals.dtype == np.float64 and tallvals.flags.c_contiguous
        _check(lib().orc_compute_tdistrib(self._h, iseed, _dp(tallvals), tallvals.size))

    def tdistrib_batch(self, seeds, nthreads: int = 0) -> np.ndarray:
        seeds = np.ascontiguousarray(seeds, np.int32)
        out = np.zeros(seeds.size * self.neigv, np.float64)
        _check(lib().orc_tdistrib_batch(self._h, seeds.ctypes.data_as(C.POINTER(C.c_int32)),
                                        seeds.size, _dp(out), nthreads))
        return out


def rand_normal(n: int, seed: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    lib().orc_rand_normal(_dp(out), n, seed)
    return out


def randi_ansic(n: int, seed: int) -> np.ndarray:
    out = np.zeros(n, np.int32)
    lib().orc_randi_ansic(out.ctypes.data_as(C.POINTER(C.c_int32)), n, seed)
    return out


def inverse_complex(a: np.ndarray) -> np.ndarray:
    """inverse_complex, src/base_utils.f90:235-274 (zgetrf + zgetri)."""
    f = np.asfortranarray(a, np.complex128).copy(order="F")
    _check(lib().orc_inverse_complex(f.ctypes.data, f.shape[0]))
    return f


def singular_values(a: np.ndarray) -> np.ndarray:
    """singular_values, src/base_utils.f90:341-380 (zgesvd 'N','N')."""
    f = np.asfortranarray(a, np.complex128).copy(order="F")
    m, n = f.shape
    s = np.zeros(min(m, n), np.float64)
    _check(lib().orc_singular_values(f.ctypes.data, m, n, _dp(s)))
    return s


def block_tridiag(amat: np.ndarray, bdiag: np.ndarray, imat: np.ndarray) -> np.ndarray:
    """solve_block_tridiag, src/base_utils.f90:296-335: amat (nb, m, m),
    bdiag (m,), imat (nb, m, k) -> xmat (nb, m, k)."""
    nb, m, _ = amat.shape
    k = imat.shape[2]
    a = np.ascontiguousarray(np.asarray(amat, np.complex128).transpose(0, 2, 1))
    b = np.ascontiguousarray(bdiag, np.complex128)
    i = np.ascontiguousarray(np.asarray(imat, np.complex128).transpose(0, 2, 1))
    x = np.zeros_like(i)
    _check(lib().orc_block_tridiag(a.ctypes.data, b.ctypes.data, i.ctypes.data, nb, m, k, x.ctypes.data))
    return x.transpose(0, 2, 1).copy()


def diagonalize_ahca(a: np.ndarray):
    """diagonalize_ahca, src/base_utils.f90:394-444 (zgesvd 'N','A'): (T, U)."""
    f = np.asfortranarray(a, np.complex128).copy(order="F")
    m, n = f.shape
    T = np.zeros(n, np.float64)
    U = np.zeros((n, n), np.complex128, order="F")
    _check(lib().orc_diagonalize_ahca(f.ctypes.data, m, n, _dp(T), U.ctypes.data))
    return T, U


def histogram(samples, bins):
    """histogram, src/base_utils.f90:491-516 -> (histo, missing)."""
    samples = np.ascontiguousarray(samples, np.float64)
    bins = np.ascontiguousarray(bins, np.float64)
    h = np.zeros(bins.size - 1, np.float64)
    miss = C.c_double(0)
    _check(lib().orc_histogram(_dp(samples), samples.size, _dp(bins), bins.size - 1, _dp(h), C.byref(miss)))
    return h, miss.value


def prepare_distrib(tallvals, nbins: int):
    """prepare_distrib, src/main.f90:223-251 -> (rho_data (nbins, 2), missing)."""
    tallvals = np.ascontiguousarray(tallvals, np.float64)
    rho = np.zeros((2, nbins), np.float64)
    miss = C.c_double(0)
    _check(lib().orc_prepare_distrib(_dp(tallvals), tallvals.size, nbins, _dp(rho), C.byref(miss)))
    return rho.T.copy(), miss.value


def chebyshev_bins(nbins: int, xmin: float = 0.0, xmax: float = 1.0) -> np.ndarray:
    """Chebyshev-node edges, src/main.f90:233 and src/plot_histogram.f90:84."""
    import math

    return np.array([xmin + (xmax - xmin) * (1.0 - math.cos(math.pi * (i - 1) / nbins)) / 2
                     for i in range(1, nbins + 2)], np.float64)


def linear_bins(nbins: int, xmin: float = 0.0, xmax: float = 1.0) -> np.ndarray:
    """Linear edges, src/plot_histogram.f90:82."""
    i = np.arange(1, nbins + 2, dtype=np.float64)
    return xmin + (xmax - xmin) * (i - 1) / nbins
