"""Sharding of one pass over several ranks (host logic).

The drawables of a scene are split into contiguous ranges, one per rank;
each rank culls its range against the shared view and knows, per StateSet,
how many of its drawables are visible.  The only exchange is an all-gather
of those per-StateSet counts; from it every rank derives where its visible
commands go inside each StateSet region:

    dst(rank, s) = offsets[s] + sum_{r < rank} count[r][s]

so the merged buffer equals the single-rank pass bit for bit (ascending
drawable order inside each region, as in the single-rank compaction).
Every machine this package runs on has one GPU, so multi-GPU runs use
independent replicas; this module is exercised by CPU ranks (gloo).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, world_size: int, rank: int) -> tuple:
    per = (n + world_size - 1) // world_size
    lo = min(n, rank * per)
    return lo, min(n, lo + per)


def local_offsets(offsets: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """StateSet offsets of the shard [lo, hi), relative to lo."""
    return (np.clip(offsets.astype(np.int64), lo, hi) - lo).astype(np.uint32)


def placement(counts_all: np.ndarray, offsets: np.ndarray, rank: int) -> np.ndarray:
    """counts_all [world, S]: destination of rank's first visible command in
    every StateSet region."""
    before = counts_all[:rank].sum(axis=0) if rank else np.zeros(counts_all.shape[1], np.int64)
    return offsets[:-1].astype(np.int64) + before


def exchange_counts(local_counts: np.ndarray, group=None) -> np.ndarray:
    """All-gather of the per-StateSet counts (torch.distributed)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(local_counts.astype(np.int64))
    out = [torch.zeros_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return torch.stack(out).numpy()
