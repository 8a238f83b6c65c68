"""Several GPUs as replicas: one process per GPU, realizations sharded by seed.

Realizations are independent (src/main.f90:134-179 runs them as an OpenMP
loop over seeds), so the seed loop splits into contiguous seed ranges with
no exchange during the sweep.  The only collective steps are at the end:
the sum of the histogram counts (the histogram of the union is the sum of
the per-rank histograms on the same edges), the gather of the raw
eigenvalues when they are saved, and the max-over-ranks time.  Any
torch.distributed backend works (NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations

import numpy as np


def seed_range(rank: int, world: int, nseed: int) -> np.ndarray:
    """Seeds of `rank` when seeds 1..nseed are split over `world` ranks:
    contiguous and balanced (the first nseed % world ranks take one more)."""
    if world < 1 or not 0 <= rank < world or nseed < 0:
        raise ValueError(f"invalid split: rank {rank} of {world}, {nseed} seeds")
    base, extra = divmod(nseed, world)
    start = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return np.arange(start + 1, start + count + 1, dtype=np.int32)


def _device(group):
    import torch.distributed as dist

    return "cuda" if dist.get_backend(group) == "nccl" else "cpu"


def sum_counts(histo: np.ndarray, missing: float, group=None) -> tuple[np.ndarray, float]:
    """Histogram counts (and the missing count) summed over the ranks.
    Counts are integers held in float64, so the sum is exact below 2^53."""
    import torch
    import torch.distributed as dist

    buf = torch.tensor(np.append(np.asarray(histo, np.float64), missing), dtype=torch.float64,
                       device=_device(group))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.cpu().numpy()
    return out[:-1], float(out[-1])


def gather_values(values: np.ndarray, group=None) -> np.ndarray:
    """The concatenation of every rank's values in rank order (ranks may
    hold different lengths), on every rank."""
    import torch
    import torch.distributed as dist

    dev = _device(group)
    world = dist.get_world_size(group)
    n = torch.tensor([len(values)], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(s.item()) for s in sizes]
    width = max(sizes) if sizes else 0
    buf = torch.zeros(width, dtype=torch.float64, device=dev)
    buf[: len(values)] = torch.as_tensor(np.asarray(values, np.float64), device=dev)
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    return np.concatenate([p[:s].cpu().numpy() for p, s in zip(parts, sizes)])


def max_over_ranks(x: float, group=None) -> float:
    """The largest value over the ranks (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
