"""Oracle fixtures for the large-mode parity checks (test infrastructure).

At 512 modes on a 2048-point grid the oracle (the reference's algorithm with
LAPACK, one core) needs ~0.2 s per slice, i.e. minutes to an hour per seed,
which is too slow to run inside a GPU test.  This script runs it once on
the CPU and stores, per seed,
  * the neigv transmission eigenvalues T_n (descending, as zgesvd gives them),
  * ||t||_F of the filtered Fisher-Lee t, and
  * a sketch t @ V of t with K fixed complex Gaussian probe vectors V
    (numpy default_rng(SKETCH_SEED)), from which a test estimates the
    relative Frobenius error of its own t without storing t itself:
    for Gaussian V, ||D V||_F^2 / K is an unbiased estimate of ||D||_F^2.

Configurations:
  c5       N = M = 512 (kW/pi = 512.5), Nx = 10^4, ny = 2048, L/l_s = 20,
           eps = 0, seeds 1..16: the large diffusive sweep, whose smallest
           eigenvalues (closed channels, T ~ exp(-2L/xi)) reach ~1e-12;
  c5short  the same guide with Nx = 2000 slices (same L/l_s, so the same
           spread of T), seeds 1..2: sized for a GPU test.

  c3top8   the 8 costliest guides (M^3 Nx) of the batched-uneven workload
           (bench.uneven_items: all N = 256, Nx ~ 4900-5000, three absorbing,
           which takes the complex sqrt(mu) branch of Fisher-Lee), each with
           its own seed;
  difffd   the differentiation guide (M = 128, kW/pi = 128.5, Nx = 1000,
           ny = 512, L/l_s = 5), seeds 1 and 2, 64 random grid cells each
           (numpy default_rng(1000 + seed)): central finite differences of
           L1 = Tr(t^H t) and L2 = Tr((t^H t)^2) from the oracle, for the
           adjoint gradient test, at the step 1e-6 sigma_U and, as a reference
           with less rounding noise, Richardson-extrapolated from the steps
           64e-6 and 128e-6 sigma_U: (4 D(h) - D(2h)) / 3 cancels the h^2 term
           (the oracle's rounding noise in D falls as 1/h: ~1e-5 of the
           largest value at 1e-6 sigma_U, ~2e-7 at 64e-6 sigma_U; the h^4
           term left is below 1e-7).

Usage:  python tests/golden/make_large_fixtures.py c5short [--threads 2]
        python tests/golden/make_large_fixtures.py c5 [--threads 8]
        python tests/golden/make_large_fixtures.py c3top8 [--threads 8]
        python tests/golden/make_large_fixtures.py difffd [--threads 8]
Items run in parallel threads (the oracle's C calls release the GIL).
"""
from __future__ import annotations

import argparse
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

SKETCH_SEED = 20261204
SKETCH_K = 4

CONFIGS = {
    "c5": dict(kw=dict(boundtype="dirichlet", nxdiso=10000, nxfree=0, wol=256.25, exfac=1.0, aratio=1.0,
                       dscat=20.0, ny=2048), seeds=list(range(1, 17))),
    "c5short": dict(kw=dict(boundtype="dirichlet", nxdiso=2000, nxfree=0, wol=256.25, exfac=1.0, aratio=1.0,
                            dscat=20.0, ny=2048), seeds=[1, 2]),
}


DIFF_KW = dict(boundtype="dirichlet", nxdiso=1000, nxfree=0, wol=64.25, exfac=1.0, aratio=1.0, dscat=5.0, ny=512)
DIFF_SEEDS = (1, 2)
DIFF_CELLS = 64


def c3_top8():
    """(kw, seed) of the 8 costliest guides of the batched-uneven workload."""
    import bench

    items = bench.uneven_items()
    cost = sorted((int(2 * kw["wol"]) ** 3 * kw["nxdiso"], k) for k, (kw, _) in enumerate(items))
    return [items[k] for _, k in cost[-8:]]


def diff_cells(seed: int, nxdiso: int, ny: int) -> np.ndarray:
    rng = np.random.default_rng(1000 + seed)
    return np.stack([rng.integers(0, nxdiso, DIFF_CELLS), rng.integers(0, ny, DIFF_CELLS)], axis=1)


def losses(t: np.ndarray) -> tuple[float, float]:
    A = t.conj().T @ t
    return float(np.sum(np.abs(t) ** 2)), float(np.sum(np.abs(A) ** 2))


def sketch_vectors(ncol: int) -> np.ndarray:
    rng = np.random.default_rng(SKETCH_SEED)
    return (rng.standard_normal((ncol, SKETCH_K)) + 1j * rng.standard_normal((ncol, SKETCH_K))) / np.sqrt(2.0)


def path(name: str) -> str:
    return os.path.join(HERE, f"oracle_{name}.npz")


def make_c3(threads: int) -> None:
    import oracle as O

    items = c3_top8()

    def one(it):
        kw, seed = it
        o = O.Waveguide(**kw)
        t0 = time.time()
        T, t = o.tdistrib_upot(o.potential(seed), want_t=True)
        print(f"seed {seed}: {time.time() - t0:.0f} s, T_min={T.min():.3e}", flush=True)
        return seed, T, np.linalg.norm(t), t @ sketch_vectors(t.shape[1])

    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, items))
    np.savez(path("c3top8"), seeds=np.array([r[0] for r in res], np.int32), T=np.stack([r[1] for r in res]),
             tnorm=np.array([r[2] for r in res]), sketch=np.stack([r[3] for r in res]), sketch_seed=SKETCH_SEED,
             params=np.array(repr([kw for kw, _ in items])))
    print("wrote", path("c3top8"))


def make_diff(threads: int) -> None:
    import oracle as O

    o = O.Waveguide(**DIFF_KW)
    h = 1e-6 * o.stdu
    jobs = []
    pots = {s: o.potential(s) for s in DIFF_SEEDS}
    for s in DIFF_SEEDS:
        for c, (ix, iy) in enumerate(diff_cells(s, o.nxdiso, o.ny)):
            jobs.append((s, c, int(ix), int(iy)))

    def central(s, ix, iy, step):
        up, um = pots[s].copy(), pots[s].copy()
        up[iy, ix] += step
        um[iy, ix] -= step
        lp = losses(o.tdistrib_upot(up, want_t=True)[1])
        lm = losses(o.tdistrib_upot(um, want_t=True)[1])
        return np.array([(lp[0] - lm[0]) / (2 * step), (lp[1] - lm[1]) / (2 * step)])

    def one(job):
        s, c, ix, iy = job
        d1, d64, d128 = (central(s, ix, iy, m * h) for m in (1, 64, 128))
        return s, c, d1, (4 * d64 - d128) / 3

    t0 = time.time()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, jobs))
    fd = np.zeros((len(DIFF_SEEDS), DIFF_CELLS, 2))
    fdr = np.zeros_like(fd)
    for s, c, d1, dr in res:
        fd[DIFF_SEEDS.index(s), c] = d1
        fdr[DIFF_SEEDS.index(s), c] = dr
    L = np.array([losses(o.tdistrib_upot(pots[s], want_t=True)[1]) for s in DIFF_SEEDS])
    cells = np.stack([diff_cells(s, o.nxdiso, o.ny) for s in DIFF_SEEDS])
    np.savez(path("difffd"), seeds=np.array(DIFF_SEEDS, np.int32), cells=cells, fd=fd, fd_rich=fdr, losses=L,
             step=h, params=np.array(repr(DIFF_KW)))
    print("spec-step FD vs extrapolated, max |diff| / max |FD| per loss:",
          np.max(np.abs(fd - fdr), axis=(0, 1)) / np.max(np.abs(fdr), axis=(0, 1)))
    print(f"wrote {path('difffd')} in {time.time() - t0:.0f} s")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=sorted(CONFIGS) + ["c3top8", "difffd"])
    ap.add_argument("--threads", type=int, default=2)
    ap.add_argument("--seeds", type=str, default="", help="comma-separated subset (default: the config's)")
    args = ap.parse_args()
    import oracle as O

    if args.config == "c3top8":
        return make_c3(args.threads)
    if args.config == "difffd":
        return make_diff(args.threads)
    cfg = CONFIGS[args.config]
    seeds = [int(s) for s in args.seeds.split(",")] if args.seeds else cfg["seeds"]
    o = O.Waveguide(**cfg["kw"])

    def one(seed: int):
        t0 = time.time()
        T, t = o.tdistrib_upot(o.potential(seed), want_t=True)
        V = sketch_vectors(t.shape[1])
        print(f"seed {seed}: {time.time() - t0:.0f} s, T_min={T.min():.3e}", flush=True)
        return seed, T, np.linalg.norm(t), t @ V

    with ThreadPoolExecutor(max_workers=args.threads) as ex:
        res = sorted(ex.map(one, seeds))
    np.savez(path(args.config), seeds=np.array([r[0] for r in res], np.int32),
             T=np.stack([r[1] for r in res]), tnorm=np.array([r[2] for r in res]),
             sketch=np.stack([r[3] for r in res]), sketch_seed=SKETCH_SEED,
             params=np.array(repr(cfg["kw"])))
    print("wrote", path(args.config))


if __name__ == "__main__":
    main()
