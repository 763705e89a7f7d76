"""Plain pass on the GPU against the oracle and the golden fixtures: world
matrices, visible sets, LOD picks, per-StateSet counts, every command word
and the marginal bitmask must match bit for bit."""
import hashlib
import json
import os

import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same, bits, gpu_cull, scene_from_npz
from oracle import bind

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_small_golden_fixture(ctx):
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    sc = scene_from_npz(g)
    res, ds, _ = gpu_cull(ctx, sc, want_world=True)
    assert np.array_equal(res["counts"], g["counts"])
    v = bind.valid_cmds(res["cmds"], res["counts"], sc.state_set_offsets).view(np.uint32).reshape(-1, 5)
    assert np.array_equal(v, g["valid_cmds"])
    assert np.array_equal(res["marginal"], g["marginal"])
    assert np.array_equal(bits(res["world"]), bits(g["world"]))


def test_c1_against_golden_and_oracle(ctx):
    d = json.load(open(os.path.join(GOLDEN, "c1.json")))
    sc = scenes.config1()
    assert sha(sc.local) == d["inputs"]["local"]          # the generator reproduces on this machine
    res, _, _ = gpu_cull(ctx, sc, want_world=True)
    assert res["counts"].tolist() == d["outputs"]["counts"]
    assert sha(bind.valid_cmds(res["cmds"], res["counts"], sc.state_set_offsets)) == d["outputs"]["valid_cmds"]
    assert sha(res["marginal"]) == d["outputs"]["marginal"]
    assert sha(res["world"]) == d["outputs"]["world"]
    ref = bind.cull(sc, sc.views[0], want_world=True)
    assert_same(res, ref, sc.state_set_offsets)


@pytest.mark.parametrize("n,levels,S,lods,empty", [
    (1, 0, 1, 1, ()), (31, 1, 2, 2, ()), (32, 2, 3, 3, (1,)), (2047, 2, 5, 4, ()),
    (2048, 1, 4, 3, (0, 3)), (2049, 3, 7, 3, (6,)), (5000, 2, 1, 2, ()), (100_003, 3, 64, 3, (5, 17)),
    (40_000, 2, 3000, 3, ()), (70_001, 0, 9, 1, (8,)),
    # Edges of a warp's 256 drawables, and more StateSets than
    # the 4,096 offsets staged in shared memory.
    (255, 1, 2, 2, ()), (256, 2, 3, 3, (2,)), (257, 1, 300, 3, ()), (300_001, 2, 5000, 3, (7, 4999)),
])
def test_edge_cases_against_oracle(ctx, n, levels, S, lods, empty):
    sc = scenes.small_scene(seed=n + 7 * levels, n=n, num_levels=levels, num_state_sets=S, num_lods=lods,
                            empty_state_sets=empty, fanout=3)
    res, _, _ = gpu_cull(ctx, sc, want_world=True)
    ref = bind.cull(sc, sc.views[0], want_world=True)
    assert_same(res, ref, sc.state_set_offsets)
    for s in empty:
        assert res["counts"][s] == 0


def test_marginal_band_against_oracle(ctx):
    """Spheres placed against the six planes at surface distances around
    the 1e-5 band: about a quarter are marginal.  Visibility, LOD, every
    command word and every marginal bit equal the oracle's."""
    sc = scenes.band_scene(seed=5, n=200_003)
    res, _, _ = gpu_cull(ctx, sc, want_world=True)
    ref = bind.cull(sc, sc.views[0], want_world=True)
    assert_same(res, ref, sc.state_set_offsets)
    marked = int(np.unpackbits(res["marginal"].view(np.uint8)).sum())
    assert 0.15 * sc.n < marked < 0.35 * sc.n


def test_empty_scene(ctx):
    sc = scenes.small_scene(seed=1, n=0, num_levels=1, num_state_sets=4, num_lods=2)
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, 0, 4)
    ctx.upload(out.counts, np.full(4, 99, np.uint32))
    ds.cull(sc.views[0], out)
    ctx.sync()
    assert ctx.download(out.counts, np.uint32, (4,)).tolist() == [0, 0, 0, 0]


def test_repeat_passes_are_identical(ctx):
    """The lookback control block re-arms itself: back-to-back passes (no
    memset in between) give the same bits."""
    sc = scenes.config2(n=1 << 18)
    ds = lib.DeviceScene(ctx, sc)
    outs = [lib.CullOutputs(ctx, sc.n, sc.num_state_sets) for _ in range(3)]
    for o in outs:
        ds.cull(sc.views[0], o)
    ctx.sync()
    ctx.check_device_error()
    r = [o.fetch() for o in outs]
    ref = bind.cull(sc, sc.views[0])
    for x in r:
        assert_same(x, ref, sc.state_set_offsets)


def test_c3_deep_hierarchy_against_oracle(ctx):
    sc = scenes.config3(n=1 << 19)
    res, _, _ = gpu_cull(ctx, sc, want_world=True)
    ref = bind.cull(sc, sc.views[0], want_world=True)
    assert_same(res, ref, sc.state_set_offsets)


def test_c3_full_size_against_oracle(ctx):
    """The deep-hierarchy scene at its stated size: 4,194,304 drawables
    under 8 internal levels (branching U{2..16}); counts, every command
    word, the marginal bitmask and all world matrices compared in full.
    Frame timing reports one time per propagated level."""
    sc = scenes.config3()
    assert sc.n == 4_194_304 and len(sc.level_sizes) == 8
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ctx.collect_frame_info(True)
    ds.cull(sc.views[0], out)
    ctx.sync()
    frames = ctx.frame_infos(with_levels=True)
    ctx.collect_frame_info(False)
    ctx.check_device_error()
    res = out.fetch()
    res["world"] = ctx.download(ds.buffers().world, np.float32, (sc.n, 16))
    ref = bind.cull(sc, sc.views[0], threads=bind.max_threads(), want_world=True)
    assert_same(res, ref, sc.state_set_offsets)
    # Levels 1-3 (2 + 24 + 216 nodes, with level 0's one node within the
    # 256 of the folded launch) run in one launch, whose time frame timing
    # gives to level 1.
    lv = frames[0][4]
    assert len(frames) == 1 and len(lv) == 7
    assert lv[0] > 0 and all(t >= 0 for t in lv) and all(t > 0 for t in lv[3:])
    assert sum(lv) <= frames[0][0] * 1.01 + 1e-3
    assert ctx.launch_count > 0


@pytest.mark.parametrize("n,levels,fanout", [
    (40_000, 6, 4),    # levels 1-2 folded (with level 0: 9 + 39 + 156 nodes), 3-5 launched one by one
    (400, 4, 3),       # every internal level folded (14 + 44 + 133 nodes)
    (200_000, 8, 4),   # levels 1-2 folded (3 + 12 + 48 nodes), then five level kernels
])
def test_folded_levels_against_oracle(ctx, n, levels, fanout):
    sc = scenes.small_scene(seed=n + levels, n=n, num_levels=levels, num_state_sets=7, num_lods=3, fanout=fanout)
    res, ds, _ = gpu_cull(ctx, sc, want_world=True)
    ref = bind.cull(sc, sc.views[0], want_world=True)
    assert_same(res, ref, sc.state_set_offsets)
    # Every level's world matrices, folded or not: level l from the GPU's
    # level l-1 by the oracle's product (the first 4,096 nodes per level).
    b = ds.buffers()
    prev = None
    for l, (loc, par) in enumerate(zip(sc.level_local, sc.level_parent)):
        got = ctx.download(b.level_world[l], np.float32, loc.shape)
        if l:
            k = min(len(par), 4096)
            want = np.stack([bind.mat4_mul(prev[int(par[i])], loc[i]) for i in range(k)])
            assert np.array_equal(bits(got[:k]), bits(want)), l
        prev = got
    assert ctx.check_device_error() == 0


def test_bad_parent_in_a_folded_level_is_reported(ctx):
    sc = scenes.small_scene(seed=4, n=3_000, num_levels=5, num_state_sets=3, fanout=3)
    sc.level_parent = list(sc.level_parent)
    sc.level_parent[2] = sc.level_parent[2].copy()
    sc.level_parent[2][1] = 1_000_000
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(sc.views[0], out)
    st, bits_ = ctx.device_error_status()
    assert st == lib.DEVICE and bits_ & 0x4


def test_c2_full_size_against_oracle(ctx):
    """The headline scene: 16,777,216 drawables, compared in full."""
    sc = scenes.config2()
    res, _, _ = gpu_cull(ctx, sc)
    ref = bind.cull(sc, sc.views[0])
    assert_same(res, ref, sc.state_set_offsets)
    frac = res["counts"].sum() / sc.n
    assert 0.2 <= frac <= 0.4


def test_tile_scan_spans_chunks(ctx):
    """More tiles than the tile scan takes in one chunk (8,192 tiles of
    2,048 drawables), with three StateSets, so regions carry their counts
    across the chunk boundary, and a ragged last tile."""
    sc = scenes.config2(n=20_000_001, num_state_sets=3)
    res, _, _ = gpu_cull(ctx, sc)
    ref = bind.cull(sc, sc.views[0])
    assert_same(res, ref, sc.state_set_offsets)


def test_upload_after_cull_is_ordered(ctx):
    """A frame loop without synchronisation: cull, upload the next frame's
    inputs into the same scene from pinned memory, cull again.  The first
    pass must see the old inputs and the second the new ones: the upload
    waits for the first pass, the second pass for the upload."""
    import dataclasses
    a = scenes.config2(n=1 << 22, seed=1)
    b = scenes.config2(n=1 << 22, seed=2)
    # The second frame: b's per-drawable and level inputs over a's
    # StateSets and LOD table (the uploads below leave those).
    ab = dataclasses.replace(a, level_local=b.level_local, level_parent=b.level_parent, local=b.local,
                             parent=b.parent, sphere=b.sphere, geometry=b.geometry)
    view = a.views[0]
    ref1, ref2 = bind.cull(a, view), bind.cull(ab, view)
    pin = {}
    for name in ("local", "parent", "sphere", "geometry"):
        arr = getattr(b, name)
        pb = lib.PinnedBuffer(arr.nbytes)
        pb.view(arr.dtype, arr.shape)[...] = arr
        pin[name] = pb
    lv = []
    for loc, par in zip(b.level_local, b.level_parent):
        pl = lib.PinnedBuffer(loc.nbytes)
        pl.view(loc.dtype, loc.shape)[...] = loc
        pp = None
        if par is not None:
            pp = lib.PinnedBuffer(par.nbytes)
            pp.view(par.dtype, par.shape)[...] = par
        lv.append((pl, pp, loc.shape[0]))
    ds = lib.DeviceScene(ctx, a)
    ctx.sync()
    out1 = lib.CullOutputs(ctx, a.n, a.num_state_sets)
    out2 = lib.CullOutputs(ctx, a.n, a.num_state_sets)
    L = ctx.lib
    ds.cull(view, out1)
    for l, (pl, pp, n_l) in enumerate(lv):
        lib.check(L.cadr_scene_upload_level(ds.handle, l, pl.ptr, pp.ptr if pp else None, 0, n_l))
    lib.check(L.cadr_scene_upload_drawables(ds.handle, pin["local"].ptr, pin["parent"].ptr, pin["sphere"].ptr,
                                            pin["geometry"].ptr, 0, a.n))
    ds.cull(view, out2)
    ctx.sync()
    assert_same(out1.fetch(), ref1, a.state_set_offsets)
    assert_same(out2.fetch(), ref2, a.state_set_offsets)


def test_staged_upload_path_equals_pinned(ctx):
    """Host inputs from pageable memory go through the pinned ring on the
    side stream; from pinned memory they are copied directly: same result."""
    sc = scenes.config2(n=1 << 16)
    res_a, _, _ = gpu_cull(ctx, sc)
    pin = lib.PinnedBuffer(sc.local.nbytes)
    arr = pin.view(np.float32, sc.local.shape)
    arr[...] = sc.local
    sc2 = scenes.Scene(sc.name, sc.seed, sc.level_local, sc.level_parent, arr, sc.parent, sc.sphere,
                       sc.geometry, sc.state_set_offsets, sc.lods, sc.num_lods, sc.views)
    res_b, _, _ = gpu_cull(ctx, sc2)
    assert_same(res_a, res_b, sc.state_set_offsets)


def test_bad_parent_index_is_reported(ctx):
    sc = scenes.small_scene(seed=3, n=5000, num_levels=2, num_state_sets=3)
    sc.parent = sc.parent.copy()
    sc.parent[17] = 10_000_000
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(sc.views[0], out)
    st, bits_ = ctx.device_error_status()
    assert st == lib.DEVICE and bits_ & 0x4
    # the context stays usable
    res, _, _ = gpu_cull(ctx, scenes.small_scene(seed=3, n=5000, num_levels=2, num_state_sets=3))
    assert res["counts"].sum() > 0


def test_download_commands_reads_the_valid_prefixes(ctx):
    """cadr_download_commands copies exactly each region's valid commands
    to the same index of host memory (touching ranges merged), leaves the
    rest alone, and rejects a count larger than its region."""
    import ctypes
    sc = scenes.small_scene(seed=21, n=50_000, num_levels=2, num_state_sets=40, num_lods=3, empty_state_sets=(3, 4))
    res, ds, out = gpu_cull(ctx, sc)
    counts = np.ascontiguousarray(res["counts"], np.uint32)
    offs = np.ascontiguousarray(sc.state_set_offsets, np.uint32)
    host = lib.PinnedBuffer(sc.n * 20)
    h = host.view(np.uint8, (sc.n * 20,))
    h[:] = 0xAB
    nbytes = ctypes.c_uint64()
    lib.check(ctx.lib.cadr_download_commands(ctx.handle, host.ptr, out.cmds.ptr, counts.ctypes.data, offs.ctypes.data,
                                             sc.num_state_sets, ctypes.byref(nbytes), None))
    ctx.sync()
    assert nbytes.value == 20 * int(counts.sum())
    got = host.view(scenes.CMD_DTYPE, (sc.n,))
    valid = np.zeros(sc.n, bool)
    for s_ in range(sc.num_state_sets):
        valid[offs[s_]:offs[s_] + counts[s_]] = True
    assert np.array_equal(bits(got[valid]), bits(res["cmds"][valid]))
    assert (h.reshape(sc.n, 20)[~valid] == 0xAB).all()
    bad = counts.copy()
    bad[0] = offs[1] - offs[0] + 1
    assert ctx.lib.cadr_download_commands(ctx.handle, host.ptr, out.cmds.ptr, bad.ctypes.data, offs.ctypes.data,
                                          sc.num_state_sets, None, None) == lib.INVALID_ARG


def test_stream_mix_probe_measures_bandwidth(ctx):
    """cadr_measure_stream_mix (the bench's same-traffic ceiling) runs and
    returns a bandwidth, and rejects an empty size."""
    gbs = ctx.measure_stream_mix(1 << 22, 3)
    assert 100.0 < gbs < 20_000.0
    with pytest.raises(lib.CadrError):
        ctx.measure_stream_mix(0, 3)
