"""Replicas on several GPUs (one process per GPU, seeds sharded), tested on
the host with two gloo ranks: the seed split, the summed histogram counts,
the gathered eigenvalues and the max-over-ranks time must equal what one
process computes for all seeds.  The per-seed eigenvalues are stand-ins
(deterministic per seed); the histogram is the oracle's."""
import os
import socket

import numpy as np
import pytest

import oracle as O
from recurgreen_gb300 import replicas
from recurgreen_gb300.tdistrib import chebyshev_bins, density_from_counts

NSEED, NBINS, PER_SEED = 13, 40, 6


def _stand_in(seed: int) -> np.ndarray:
    """One realization's eigenvalues, as values in [0, 1) fixed by the seed."""
    return np.sort(np.random.default_rng(seed).random(PER_SEED))[::-1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = replicas.seed_range(rank, world, NSEED)
    local = np.concatenate([_stand_in(int(s)) for s in seeds]) if seeds.size else np.zeros(0)
    bins = chebyshev_bins(NBINS)
    h, miss = O.histogram(local, bins) if local.size else (np.zeros(NBINS), 0.0)
    hs, ms = replicas.sum_counts(h, miss)
    allv = replicas.gather_values(local)
    tmax = replicas.max_over_ranks(0.5 + rank)
    queue.put((rank, hs, ms, allv, tmax))
    dist.barrier()
    dist.destroy_process_group()


def test_seed_range_partitions():
    for nseed in (0, 1, 7, 100, 4096):
        for world in (1, 2, 3, 8):
            parts = [replicas.seed_range(r, world, nseed) for r in range(world)]
            np.testing.assert_array_equal(np.concatenate(parts), np.arange(1, nseed + 1))
            sizes = [p.size for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.seed_range(2, 2, 10)


def test_two_gloo_ranks_match_one_process():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    queue = ctx.SimpleQueue()
    mp.spawn(_worker, args=(2, _free_port(), queue), nprocs=2, join=True)
    got = sorted([queue.get() for _ in range(2)], key=lambda r: r[0])
    allseeds = np.concatenate([_stand_in(s) for s in range(1, NSEED + 1)])
    bins = chebyshev_bins(NBINS)
    ref_h, ref_m = O.histogram(allseeds, bins)
    for rank, hs, ms, allv, tmax in got:
        np.testing.assert_array_equal(hs, ref_h)  # counts are exact
        assert ms == ref_m
        np.testing.assert_array_equal(allv, allseeds)  # seed order
        assert tmax == 1.5
    # the density from the summed counts is the reference's prepare_distrib of all samples
    rho = density_from_counts(got[0][1], bins)
    ref_rho, _ = O.prepare_distrib(allseeds, NBINS)
    np.testing.assert_allclose(rho, ref_rho, rtol=1e-14, atol=0)
    del torch
