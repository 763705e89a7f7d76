"""Batched form (one persistent launch over (view, tile) items, CUDA graph
replay) against the plain pass: identical visible sets and draw buffers."""
import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same
from oracle import bind

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c4_small(ctx):
    scs = scenes.config4(num_scenes=5, lo=1000, hi=150_000)
    dss = [lib.DeviceScene(ctx, sc) for sc in scs]
    for ds in dss:
        ds.propagate(world_spheres=True)
    ctx.sync()
    return scs, dss


def _plain(ctx, sc, ds, view):
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(view, out)
    ctx.sync()
    return out.fetch()


def test_world_spheres_match_oracle(ctx, c4_small):
    scs, dss = c4_small
    for sc, ds in zip(scs, dss):
        ref = bind.cull(sc, sc.views[0], want_world=True)
        b = ds.buffers()
        ws = ctx.download(b.world_sphere, np.float32, (sc.n, 4))
        assert np.array_equal(ws.view(np.uint32), ref["world_sphere"].view(np.uint32))
        ds.host  # keep alive


@pytest.mark.parametrize("tuning", [None, (128, 4, 4), (512, 8, 2), (256, 16, 8), (256, 8, 4, 1)])
def test_batched_equals_plain(ctx, c4_small, tuning):
    scs, dss = c4_small
    items, outs = [], []
    for sc, ds in zip(scs, dss):
        ds.buffers  # committed by upload_all
        for v in sc.views:
            o = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
            items.append((ds, v, o))
            outs.append((sc, ds, v, o))
    arr = lib.batch_views(items)
    t = lib.Tuning(*(tuning + (0,))[:4]) if tuning else None
    for _ in range(2):  # second call replays the captured graph
        lib.cull_batched(ctx, arr, t, use_graph=True)
        ctx.sync()
        ctx.check_device_error()
        for sc, ds, v, o in outs:
            assert_same(o.fetch(), _plain(ctx, sc, ds, v), sc.state_set_offsets)


def test_batched_against_oracle_spheres(ctx, c4_small):
    scs, dss = c4_small
    sc, ds = scs[-1], dss[-1]
    items = [(ds, v, lib.CullOutputs(ctx, sc.n, sc.num_state_sets)) for v in sc.views]
    lib.cull_batched(ctx, lib.batch_views(items), None, use_graph=False)
    ctx.sync()
    ref_full = bind.cull(sc, sc.views[0], want_world=True)
    for (_, v, o) in items:
        ref = bind.cull_spheres(ref_full["world_sphere"], sc.geometry, sc.state_set_offsets, sc.lods,
                                sc.num_lods, v)
        assert_same(o.fetch(), ref, sc.state_set_offsets)


def test_autotune_picks_a_supported_tuning(ctx, c4_small):
    scs, dss = c4_small
    items = [(ds, v, lib.CullOutputs(ctx, sc.n, sc.num_state_sets)) for sc, ds in zip(scs, dss)
             for v in sc.views[:2]]
    t, ms = lib.autotune_batched(ctx, lib.batch_views(items), reps=2)
    assert t.block_threads in (128, 256, 512) and t.items_per_thread in (4, 8, 16) and ms > 0


def test_autotune_cache_skips_timing_and_gives_identical_output(ctx, c4_small, tmp_path):
    """With a tuning cache, the second autotune of the same batch shape
    launches nothing and returns the stored pick; the batch culled with it
    equals the plain passes."""
    scs, dss = c4_small
    items, outs = [], []
    for sc, ds in zip(scs, dss):
        for v in sc.views[:3]:
            o = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
            items.append((ds, v, o))
            outs.append((sc, ds, v, o))
    arr = lib.batch_views(items)
    lib.set_tuning_cache(ctx, str(tmp_path / "tuning.json"))
    try:
        l0 = ctx.launch_count
        t1, ms1 = lib.autotune_batched(ctx, arr, reps=2)
        l1 = ctx.launch_count
        assert l1 - l0 >= 24 * 3
        t2, ms2 = lib.autotune_batched(ctx, arr, reps=2)
        assert ctx.launch_count == l1
        assert (t2.block_threads, t2.items_per_thread, t2.ctas_per_sm) == (t1.block_threads, t1.items_per_thread,
                                                                           t1.ctas_per_sm)
        assert abs(ms2 - ms1) < 1e-3
    finally:
        lib.set_tuning_cache(ctx, None)
    lib.cull_batched(ctx, arr, t2, use_graph=True)
    ctx.sync()
    ctx.check_device_error()
    for sc, ds, v, o in outs:
        assert_same(o.fetch(), _plain(ctx, sc, ds, v), sc.state_set_offsets)


def test_batched_marginal_bits_equal_plain(ctx):
    """Spheres against the planes (about a quarter inside the 1e-5 band):
    the batched form's marginal bits equal the plain pass's."""
    sc = scenes.band_scene(seed=13, n=150_001)
    ds = lib.DeviceScene(ctx, sc)
    ds.propagate(world_spheres=True)
    o = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    lib.cull_batched(ctx, lib.batch_views([(ds, sc.views[0], o)]), None, use_graph=False)
    ctx.sync()
    ctx.check_device_error()
    got, ref = o.fetch(), _plain(ctx, sc, ds, sc.views[0])
    assert_same(got, ref, sc.state_set_offsets)
    assert np.unpackbits(got["marginal"].view(np.uint8)).sum() > 0.15 * sc.n


@pytest.mark.parametrize("form", [lib.BATCHED_PERSISTENT, lib.BATCHED_THREE_LAUNCH])
def test_batch_with_empty_and_ragged_scenes(ctx, form):
    """Scenes of 0, 1, 2,047, 2,049 and 100,003 drawables (many StateSets,
    some empty) in one batch, in both forms: each view equals its plain
    pass, the empty scene's counts are zero."""
    # The last two have more StateSets than either form stages in shared
    # memory (2,048 offsets for the persistent form, 4,096 for the write
    # kernel of the three-launch form).
    shapes = [(0, 4), (1, 1), (2047, 5), (2049, 300), (100_003, 64), (30_000, 3000), (40_000, 5000)]
    items, outs = [], []
    for k, (n, S) in enumerate(shapes):
        sc = scenes.small_scene(seed=70 + k, n=n, num_levels=2 if n else 1, num_state_sets=S, num_lods=3,
                                empty_state_sets=(1,) if S > 2 else ())
        ds = lib.DeviceScene(ctx, sc)
        ds.propagate(world_spheres=True)
        for v in range(2):
            view = sc.views[0] if v == 0 else scenes.random_view(9, k)
            o = lib.CullOutputs(ctx, n, S)
            ctx.upload(o.counts, np.full(S, 77, np.uint32))
            items.append((ds, view, o))
            outs.append((sc, ds, view, o))
    lib.cull_batched(ctx, lib.batch_views(items), lib.Tuning(256, 8, 4, form), use_graph=False)
    ctx.sync()
    ctx.check_device_error()
    for sc, ds, view, o in outs:
        got = o.fetch()
        if sc.n == 0:
            assert (got["counts"] == 0).all()
            continue
        assert_same(got, _plain(ctx, sc, ds, view), sc.state_set_offsets)


def test_server_in_the_three_launch_form(ctx, c4_small):
    """The serving loop batches with the context's tuning: in the
    three-launch form its results equal the plain passes."""
    scs, dss = c4_small
    saved = ctx.get_tuning()
    ctx.set_tuning(256, 8, 4, lib.BATCHED_THREE_LAUNCH)
    try:
        srv = lib.Server(ctx, max_inflight=2, max_batch_views=8, window_ns=100_000)
        reqs = {}
        for k in range(12):
            si = k % len(scs)
            views = np.concatenate([scenes.random_view(6, 10 * k + j) for j in range(1 + k % 3)])
            reqs[srv.submit(dss[si], views)] = (si, views)
        srv.drain()
        done = {r.request_id: r for r in srv.poll()}
        assert set(done) == set(reqs)
        for rid, (si, views) in reqs.items():
            r = done[rid]
            assert r.status == lib.OK
            for v in range(len(views)):
                counts = ctx.download(r.counts[v], np.uint32, (scs[si].num_state_sets,))
                cmds = ctx.download(r.cmds[v], scenes.CMD_DTYPE, (scs[si].n,))
                ref = _plain(ctx, scs[si], dss[si], views[v:v + 1])
                assert np.array_equal(counts, ref["counts"])
                off = scs[si].state_set_offsets
                assert np.array_equal(bind.valid_cmds(cmds, counts, off).view(np.uint8),
                                      bind.valid_cmds(ref["cmds"], ref["counts"], off).view(np.uint8))
            srv.release(rid)
        srv.close()
    finally:
        ctx.set_tuning(saved.block_threads, saved.items_per_thread, saved.ctas_per_sm, saved.form)

