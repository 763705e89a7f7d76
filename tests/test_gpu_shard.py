"""The sharded plain pass through the CUDA library (cadr_cull_shard_count,
cadr_cull_shard_write): the drawables split into contiguous ranges, each
range culled as a scene of its own, the per-StateSet counts exchanged, the
commands written straight into the merged buffer.  The merged buffer must
equal cadr_cull on the whole scene byte for byte."""
import os
import socket

import numpy as np
import pytest

from cadr_gb300 import lib, multigpu, scenes
from helpers import bits
from oracle import bind

pytestmark = pytest.mark.gpu


def _single_rank(ctx, sc):
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(sc.views[0], out)
    ctx.sync()
    ctx.check_device_error()
    return out.fetch()


def _assert_merged_equal(merged_cmds, counts, ref, offsets):
    assert np.array_equal(counts, ref["counts"])
    g = bind.valid_cmds(merged_cmds, counts, offsets)
    r = bind.valid_cmds(ref["cmds"], ref["counts"], offsets)
    assert np.array_equal(bits(g), bits(r))


@pytest.mark.parametrize("n,world,S,empty", [
    (1 << 20, 3, 37, (4, 36)),        # regions crossing both shard boundaries, empty regions at the ends
    (100_003, 2, 5, ()),              # ragged tiles at both shard ends
    (5000, 4, 3000, ()),              # more regions than drawables per shard
    (2048 * 3, 3, 2, (0,)),           # shard boundaries on tile boundaries
    (60_000, 2, 5000, (7, 4999)),     # more StateSets than the write kernel stages in shared memory
])
def test_shards_merge_to_the_single_rank_pass(ctx, n, world, S, empty):
    sc = scenes.small_scene(seed=n + world, n=n, num_levels=2, num_state_sets=S, num_lods=3,
                            empty_state_sets=empty, fanout=4)
    ref = _single_rank(ctx, sc)
    oracle_ref = bind.cull(sc, sc.views[0])
    assert np.array_equal(ref["counts"], oracle_ref["counts"])
    bounds = [multigpu.shard_bounds(n, world, r) for r in range(world)]
    shards = [lib.DeviceScene(ctx, multigpu.shard_scene(sc, lo, hi)) for lo, hi in bounds]
    merged = ctx.alloc(n * 20)
    # Phase 1 on every shard, then the exchange, then phase 2: each shard's
    # write follows its own count (another shard's count on the same
    # context in between would replace it), so count and write pairwise.
    counts = [multigpu.shard_count(ctx, ds, sc.views[0]) for ds in shards]
    everyone = np.stack(counts).astype(np.int64)
    for r, ((lo, hi), ds) in enumerate(zip(bounds, shards)):
        assert np.array_equal(multigpu.shard_count(ctx, ds, sc.views[0]), counts[r])
        multigpu.shard_write(ctx, ds, multigpu.placement(everyone, sc.state_set_offsets, r), lo, merged, n)
    ctx.check_device_error()
    got = ctx.download(merged, scenes.CMD_DTYPE, (n,))
    _assert_merged_equal(got, everyone.sum(axis=0).astype(np.uint32), ref, sc.state_set_offsets)


def test_shard_marginal_bits_are_the_shards_slice(ctx):
    sc = scenes.band_scene(seed=9, n=64 * 1024)
    ref = bind.cull(sc, sc.views[0])
    want = np.unpackbits(ref["marginal"].view(np.uint8), bitorder="little")
    for lo, hi in [multigpu.shard_bounds(sc.n, 2, r) for r in range(2)]:
        ds = lib.DeviceScene(ctx, multigpu.shard_scene(sc, lo, hi))
        d_counts, d_marg = ctx.alloc(64), ctx.alloc(((hi - lo + 31) // 32) * 4)
        v = np.ascontiguousarray(sc.views[0], lib.VIEW_DTYPE)
        lib.check(ctx.lib.cadr_cull_shard_count(ds.handle, v.ctypes.data, d_counts.ptr, d_marg.ptr, None))
        m = ctx.download(d_marg, np.uint32, ((hi - lo + 31) // 32,))
        assert np.array_equal(np.unpackbits(m.view(np.uint8), bitorder="little")[:hi - lo], want[lo:hi])


def test_shard_write_needs_its_count_phase(ctx):
    sc = scenes.small_scene(seed=2, n=4000, num_levels=1, num_state_sets=3)
    ds = lib.DeviceScene(ctx, sc)
    merged = ctx.alloc(4000 * 20)
    base = ctx.to_device(np.zeros(3, np.uint32))
    st = ctx.lib.cadr_cull_shard_write(ds.handle, base.ptr, 0, merged.ptr, 4000, None)
    assert st == lib.INVALID_ARG
    assert b"count phase" in ctx.lib.cadr_last_error()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


N_TWO_PROCESS = (1 << 20) + 777


def _rank_main(rank, world, port, q):
    """One rank in a process of its own, on GPU 0 with its own context: its
    shard through the CUDA library, the counts exchanged over gloo, its
    commands written into its own copy of the merged buffer; the written
    slots go back to the test."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from cadr_gb300 import lib, multigpu, scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenes.config2(n=N_TWO_PROCESS, num_state_sets=64)
        lo, hi = multigpu.shard_bounds(sc.n, world, rank)
        ctx = lib.Context(0)
        ds = lib.DeviceScene(ctx, multigpu.shard_scene(sc, lo, hi))
        merged = ctx.alloc(sc.n * 20)
        everyone, base = multigpu.cull_sharded(ctx, ds, sc.views[0], sc.state_set_offsets, rank, lo, merged, sc.n,
                                               multigpu.exchange_counts)
        ctx.check_device_error()
        got = ctx.download(merged, scenes.CMD_DTYPE, (sc.n,))
        mine = everyone[rank]
        slots = np.concatenate([np.arange(base[s], base[s] + mine[s]) for s in range(sc.num_state_sets)])
        q.put((rank, slots, got[slots].tobytes(), everyone.sum(axis=0)))
        dist.barrier()
        ctx.close()
    finally:
        dist.destroy_process_group()


def test_two_processes_on_one_gpu_merge_to_the_single_rank_pass(ctx):
    """Both ranks run the CUDA path on GPU 0 in separate processes (no peer
    access, no kernel of one waits on the other's); the exchange is the
    gloo all-gather of the counts.  Their written slots, merged, equal the
    single-rank pass, and no slot is written twice."""
    import torch.multiprocessing as mp
    mpc = mp.get_context("spawn")
    q = mpc.Queue()
    port = _free_port()
    procs = [mpc.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = [q.get(timeout=600) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sc = scenes.config2(n=N_TWO_PROCESS, num_state_sets=64)
    ref = _single_rank(ctx, sc)
    merged = np.zeros(sc.n, scenes.CMD_DTYPE)
    seen = np.zeros(sc.n, bool)
    for _, slots, raw, total in parts:
        assert not seen[slots].any()
        seen[slots] = True
        merged[slots] = np.frombuffer(raw, scenes.CMD_DTYPE)
        assert np.array_equal(total, ref["counts"])
    _assert_merged_equal(merged, ref["counts"], ref, sc.state_set_offsets)
