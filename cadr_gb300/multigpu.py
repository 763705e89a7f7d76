"""Sharding of one pass over several ranks (host logic).

The drawables of a scene are split into contiguous ranges, one per rank;
each rank culls its range against the shared view and knows, per StateSet,
how many of its drawables are visible.  The only exchange is an all-gather
of those per-StateSet counts; from it every rank derives where its visible
commands go inside each StateSet region:

    dst(rank, s) = offsets[s] + sum_{r < rank} count[r][s]

so the merged buffer equals the single-rank pass bit for bit (ascending
drawable order inside each region, as in the single-rank compaction).

On the device the pass splits at that exchange: cadr_cull_shard_count
(propagation, cull, LOD, per-StateSet counts of the shard) and, after the
all-gather, cadr_cull_shard_write (the commands written at their merged
slots, firstInstance offset by the shard's first drawable).  shard_count,
shard_write and cull_sharded drive the two phases; exchange_counts is the
all-gather over torch.distributed.  The machines of this build have one GPU
each, so multi-GPU benchmark runs use independent replicas; the sharded
path is tested with CPU ranks (gloo, oracle) and with two processes that
share one GPU.
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


def shard_scene(sc, lo: int, hi: int):
    """The shard [lo, hi) of a scene as a scene of its own: its drawables,
    the internal levels replicated, its StateSet offsets clipped to the
    range and taken relative to lo (empty regions stay)."""
    import dataclasses
    sl = slice(lo, hi)
    return dataclasses.replace(
        sc, local=np.ascontiguousarray(sc.local[sl]),
        parent=None if sc.parent is None else np.ascontiguousarray(sc.parent[sl]),
        sphere=np.ascontiguousarray(sc.sphere[sl]), geometry=np.ascontiguousarray(sc.geometry[sl]),
        state_set_offsets=local_offsets(sc.state_set_offsets, lo, hi))


def shard_count(ctx, ds, view) -> np.ndarray:
    """Phase 1 of a shard's pass through the CUDA library
    (cadr_cull_shard_count): the shard's visible drawables per StateSet."""
    from . import lib
    S = ds.host.num_state_sets
    d_counts = ctx.alloc(max(16, S * 4))
    v = np.ascontiguousarray(view, lib.VIEW_DTYPE)
    lib.check(ctx.lib.cadr_cull_shard_count(ds.handle, v.ctypes.data, d_counts.ptr, None, None))
    return ctx.download(d_counts, np.uint32, (S,))


def shard_write(ctx, ds, dst_base: np.ndarray, first_instance: int, merged_cmds, capacity: int) -> None:
    """Phase 2 (cadr_cull_shard_write): the shard's commands into the merged
    buffer at dst_base[s] + k, firstInstance offset by first_instance."""
    from . import lib
    d_base = ctx.to_device(np.ascontiguousarray(dst_base, np.uint32))
    lib.check(ctx.lib.cadr_cull_shard_write(ds.handle, d_base.ptr, int(first_instance), lib._ptr(merged_cmds),
                                            int(capacity), None))
    ctx.sync()


def cull_sharded(ctx, ds, view, offsets: np.ndarray, rank: int, lo: int, merged_cmds, capacity: int,
                 exchange) -> tuple:
    """One rank's sharded pass: count, exchange (`exchange` maps this rank's
    [S] counts to every rank's [world, S]), place, write.  Returns (all
    ranks' counts, this rank's destination bases)."""
    mine = shard_count(ctx, ds, view)
    everyone = np.asarray(exchange(mine), np.int64)
    base = placement(everyone, offsets, rank)
    shard_write(ctx, ds, base, lo, merged_cmds, capacity)
    return everyone, base


def exchange_counts(local_counts: np.ndarray, group=None) -> np.ndarray:
    """All-gather of the per-StateSet counts (torch.distributed)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(local_counts.astype(np.int64))
    out = [torch.zeros_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return torch.stack(out).numpy()
