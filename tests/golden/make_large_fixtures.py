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

Usage:  python tests/golden/make_large_fixtures.py c5short [--threads 2]
        python tests/golden/make_large_fixtures.py c5 [--threads 8]
The seeds run in parallel threads (the oracle's C calls release the GIL).
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


def sketch_vectors(ncol: int) -> np.ndarray:
    rng = np.random.default_rng(SKETCH_SEED)
    return (rng.standard_normal((ncol, SKETCH_K)) + 1j * rng.standard_normal((ncol, SKETCH_K))) / np.sqrt(2.0)


def path(name: str) -> str:
    return os.path.join(HERE, f"oracle_{name}.npz")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=sorted(CONFIGS))
    ap.add_argument("--threads", type=int, default=2)
    ap.add_argument("--seeds", type=str, default="", help="comma-separated subset (default: the config's)")
    args = ap.parse_args()
    import oracle as O

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
