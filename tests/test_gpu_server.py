"""Serving form: continuous batching over resident scenes; each result is
the same alone (plain pass) and in the mix."""
import time

import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from oracle import bind

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def resident(ctx):
    scs = [scenes.config2(seed=4000 + i, n=n) for i, n in enumerate([10_000, 60_000, 250_000, 33_333])]
    dss = [lib.DeviceScene(ctx, sc) for sc in scs]
    for ds in dss:
        ds.propagate(world_spheres=True)
    ctx.sync()
    return scs, dss


def _fetch(ctx, res, sc, v):
    counts = ctx.download(res.counts[v], np.uint32, (sc.num_state_sets,))
    cmds = ctx.download(res.cmds[v], scenes.CMD_DTYPE, (sc.n,))
    return counts, cmds


def test_results_alone_equal_in_the_mix(ctx, resident):
    scs, dss = resident
    srv = lib.Server(ctx, max_inflight=3, max_batch_views=16, window_ns=200_000)
    reqs = {}
    for k in range(40):
        si = k % len(scs)
        nv = 1 + k % 4
        views = np.concatenate([scenes.random_view(4, 100 * k + j) for j in range(nv)])
        rid = srv.submit(dss[si], views)
        reqs[rid] = (si, views)
        if k % 7 == 0:
            time.sleep(0.0005)
    srv.drain()
    done = {}
    deadline = time.time() + 60
    while len(done) < len(reqs) and time.time() < deadline:
        for r in srv.poll():
            done[r.request_id] = r
        time.sleep(0.001)
    assert len(done) == len(reqs)
    for rid, (si, views) in reqs.items():
        r = done[rid]
        assert r.status == lib.OK and r.complete_ns >= r.submit_ns
        sc, ds = scs[si], dss[si]
        for v in range(len(views)):
            counts, cmds = _fetch(ctx, r, sc, v)
            out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
            ds.cull(views[v:v + 1], out)
            ctx.sync()
            alone = out.fetch()
            assert np.array_equal(counts, alone["counts"])
            a = bind.valid_cmds(cmds, counts, sc.state_set_offsets)
            b = bind.valid_cmds(alone["cmds"], alone["counts"], sc.state_set_offsets)
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
        srv.release(rid)
    srv.close()


def test_admission_by_memory(ctx, resident):
    scs, dss = resident
    per_view = ((scs[2].n * 20 + 255) // 256) * 256 + 1024
    srv = lib.Server(ctx, max_inflight=2, max_batch_views=4, window_ns=50_000, memory_budget=3 * per_view)
    with pytest.raises(lib.CadrError) as e:
        srv.submit(dss[2], np.concatenate([scenes.random_view(4, j) for j in range(4)]))
    assert e.value.status == lib.REJECTED
    # six one-view requests that only fit three at a time: all complete once
    # earlier results are released
    ids = [srv.submit(dss[2], scenes.random_view(4, 900 + j)) for j in range(6)]
    got = {}
    deadline = time.time() + 60
    while len(got) < len(ids) and time.time() < deadline:
        for r in srv.poll():
            assert r.status == lib.OK
            got[r.request_id] = r
            srv.release(r.request_id)
        time.sleep(0.001)
    assert sorted(got) == sorted(ids)
    srv.close()


def test_failed_batches_give_their_memory_back(ctx, resident):
    """A batch whose launch fails (CADR_FAULT_SERVER_LAUNCH: on the host,
    before anything is launched) ends its requests with CADR_ERR_CUDA and
    returns their output memory: six requests that fit three at a time all
    fail in turn, and afterwards three requests that need the whole budget
    are admitted together and complete."""
    scs, dss = resident
    per_view = ((scs[2].n * 20 + 255) // 256) * 256 + 1024
    srv = lib.Server(ctx, max_inflight=2, max_batch_views=4, window_ns=50_000, memory_budget=3 * per_view)
    ctx.set_fault(lib.FAULT_SERVER_LAUNCH)
    try:
        failed = [srv.submit(dss[2], scenes.random_view(4, 700 + j)) for j in range(6)]
        got = {}
        deadline = time.time() + 30
        while len(got) < len(failed) and time.time() < deadline:
            for r in srv.poll():
                got[r.request_id] = r
            time.sleep(0.001)
    finally:
        ctx.set_fault(lib.FAULT_NONE)
    assert sorted(got) == sorted(failed)
    assert all(r.status == lib.CUDA for r in got.values())
    for rid in failed:
        srv.release(rid)
    ids = [srv.submit(dss[2], scenes.random_view(4, 800 + j)) for j in range(3)]
    done = {}
    deadline = time.time() + 30
    while len(done) < len(ids) and time.time() < deadline:
        for r in srv.poll():
            done[r.request_id] = r
        time.sleep(0.001)
    assert sorted(done) == sorted(ids)
    assert all(r.status == lib.OK for r in done.values())
    for rid in ids:
        srv.release(rid)
    srv.close()
