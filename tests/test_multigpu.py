"""Sharded pass over two CPU ranks (gloo): shard the drawables, cull each
shard with the oracle, exchange per-StateSet counts, place, merge; the
merged commands equal the single-rank pass."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from cadr_gb300 import multigpu, scenes
    from oracle import bind
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenes.config1()
        lo, hi = multigpu.shard_bounds(sc.n, world, rank)
        sub = scenes.Scene("shard", 0, sc.level_local, sc.level_parent, sc.local[lo:hi], sc.parent[lo:hi],
                           sc.sphere[lo:hi], sc.geometry[lo:hi], multigpu.local_offsets(sc.state_set_offsets, lo, hi),
                           sc.lods, sc.num_lods, sc.views)
        o = bind.cull(sub, sub.views[0], threads=1)
        counts_all = multigpu.exchange_counts(o["counts"])
        dst = multigpu.placement(counts_all, sc.state_set_offsets, rank)
        placed = []
        for s in range(sc.num_state_sets):
            st = int(sub.state_set_offsets[s])
            for k in range(int(o["counts"][s])):
                c = o["cmds"][st + k].copy()
                c["first_instance"] += lo
                placed.append((int(dst[s]) + k, c.tobytes()))
        gathered = [None] * world
        dist.all_gather_object(gathered, (placed, counts_all.sum(axis=0).tolist()))
        if rank == 0:
            q.put(gathered)
    finally:
        dist.destroy_process_group()


def test_two_rank_shard_merge_equals_single_rank(oracle_lib):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from cadr_gb300 import scenes
    from oracle import bind
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sc = scenes.config1()
    ref = bind.cull(sc, sc.views[0], threads=1)
    assert gathered[0][1] == ref["counts"].tolist()
    merged = {}
    for placed, _ in gathered:
        for slot, raw in placed:
            assert slot not in merged
            merged[slot] = raw
    for s in range(sc.num_state_sets):
        st = int(sc.state_set_offsets[s])
        for k in range(int(ref["counts"][s])):
            assert merged[st + k] == ref["cmds"][st + k].tobytes()
