"""Device-resident StateSet packing (cadr_pack_*) against the oracle's
restatement of StateSet::recordToCommandBuffer, bit for bit, and Tier A
run end to end on the packed array."""
import numpy as np
import pytest

from cadr_gb300 import lib, tier_a
from helpers import pack_layout_from_packed
from oracle import bind

pytestmark = pytest.mark.gpu


def random_records(n, seed):
    raw = np.random.default_rng(seed).integers(0, 2**63, size=(n, 6), dtype=np.uint64)
    return raw.view(tier_a.DRAWABLE_DTYPE).reshape(n)


def make_counts(S, n, seed, empty=()):
    rs = np.random.default_rng(seed)
    w = rs.random(S) + 0.05
    for e in empty:
        w[e] = 0.0
    counts = np.floor(w / w.sum() * n).astype(np.int64)
    counts[int(np.argmax(w))] += n - counts.sum()
    return counts


@pytest.mark.parametrize("n,S,empty", [(1, 1, ()), (1000, 7, (2, 6)), (100_003, 300, (0, 17, 299)),
                                       (2_000_000, 64, (5,))])
def test_repack_matches_oracle(ctx, n, S, empty):
    counts = make_counts(S, n, n + S, empty)
    dfs, ss, li, perm, starts = pack_layout_from_packed(counts, seed=n)
    expect = random_records(n, seed=S)
    pool = np.empty_like(expect)
    pool[np.arange(n)] = expect[perm]
    ref, ref_off = bind.pack_state_sets(dfs, ss, li, pool)
    assert np.array_equal(ref.view(np.uint8), expect.view(np.uint8))
    assert np.array_equal(ref_off, starts)
    pk = lib.Pack(ctx, n)
    pk.set_layout(dfs, ss, li)
    pk.upload(pool)
    pk.repack()
    packed, offsets = pk.fetch(tier_a.DRAWABLE_DTYPE)
    assert ctx.check_device_error() == 0
    assert np.array_equal(packed.view(np.uint8), ref.view(np.uint8))
    assert np.array_equal(offsets, ref_off)


def test_patch_dirty_rows(ctx):
    n, S = 200_000, 40
    counts = make_counts(S, n, 3)
    dfs, ss, li, perm, _ = pack_layout_from_packed(counts, seed=4)
    pool = random_records(n, seed=5)
    pk = lib.Pack(ctx, n)
    pk.set_layout(dfs, ss, li)
    pk.upload(pool)
    pk.repack()
    rs = np.random.default_rng(6)
    for rnd in range(3):
        dirty = rs.choice(n, size=n // 100, replace=False).astype(np.uint32)
        new = random_records(len(dirty), seed=100 + rnd)
        pool[dirty] = new
        pk.patch(dirty, new)
        ref, _ = bind.pack_state_sets(dfs, ss, li, pool)
        packed, _ = pk.fetch(tier_a.DRAWABLE_DTYPE)
        assert np.array_equal(packed.view(np.uint8), ref.view(np.uint8))
    # The pool took the patches too: a full repack gives the same array.
    pk.repack()
    packed2, _ = pk.fetch(tier_a.DRAWABLE_DTYPE)
    assert np.array_equal(packed2.view(np.uint8), ref.view(np.uint8))
    assert ctx.check_device_error() == 0


def test_relayout_moves_drawables(ctx):
    """A new layout (drawables moved between StateSets, lists reordered)
    over the same pool repacks to the oracle's packing of that layout."""
    n, S = 50_000, 12
    pool = random_records(n, seed=8)
    pk = lib.Pack(ctx, n)
    for seed in (9, 10):
        dfs, ss, li, _, _ = pack_layout_from_packed(make_counts(S, n, seed, (seed % S,)), seed=seed)
        pk.set_layout(dfs, ss, li)
        if seed == 9:
            pk.upload(pool)
        pk.repack()
        ref, ref_off = bind.pack_state_sets(dfs, ss, li, pool)
        packed, offsets = pk.fetch(tier_a.DRAWABLE_DTYPE)
        assert np.array_equal(packed.view(np.uint8), ref.view(np.uint8))
        assert np.array_equal(offsets, ref_off)
    assert ctx.check_device_error() == 0


@pytest.mark.parametrize("case", ["duplicate index", "index past list", "set out of range", "dfs not a permutation"])
def test_bad_layouts_are_reported(ctx, case):
    n, S = 1000, 5
    dfs, ss, li, _, _ = pack_layout_from_packed(make_counts(S, n, 1), seed=2)
    dfs, ss, li = dfs.copy(), ss.copy(), li.copy()
    if case == "duplicate index":
        k = int(np.nonzero(li == 1)[0][0])
        li[k] = 0
    elif case == "index past list":
        li[0] = n
    elif case == "set out of range":
        ss[0] = S
    else:
        dfs[1] = dfs[0]
    pk = lib.Pack(ctx, n)
    pk.set_layout(dfs, ss, li)
    pk.upload(random_records(n, seed=3))
    pk.repack()
    st, bits = ctx.device_error_status()
    assert st == lib.DEVICE and bits & lib.DEVERR_BAD_INDEX


def test_tier_a_on_packed_records(ctx):
    """Records scattered over slots, packed on the device, then
    processDrawables: the output equals the oracle on the reference's
    host-packed records, so the draws address the same data."""
    kw = dict(n=300_000, num_state_sets=24, num_geometries=4096, prims_per_geometry=3)
    probe = tier_a.build(seed=11, base=1 << 40, **kw)
    buf = ctx.alloc(probe.image.nbytes + 4096)
    im = tier_a.build(seed=11, base=buf.ptr, **kw)
    r_ind, r_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables)
    ctx.upload(buf, im.image)
    n = im.drawables.shape[0]
    dfs, ss, li, perm, starts = pack_layout_from_packed(im.state_set_counts, seed=12)
    pool = im.drawables[perm]
    pk = lib.Pack(ctx, n)
    pk.set_layout(dfs, ss, li)
    pk.upload(pool)
    pk.repack()
    packed, offsets, m = pk.buffers()
    assert m == n
    ind = ctx.alloc(n * 16)
    ptr = ctx.alloc(n * 32)
    ctx.process_drawables(im.level, im.root, packed, n, ind, ptr)
    ctx.sync()
    assert ctx.check_device_error() == 0
    assert np.array_equal(ctx.download(ind, np.uint32, (n, 4)), r_ind)
    assert np.array_equal(ctx.download(ptr, np.uint64, (n, 4)), r_ptr)
    assert np.array_equal(ctx.download(offsets, np.uint32, (len(dfs) + 1,)), starts)


def creation_order_layout(im, G):
    """Slots in drawable creation order (the order of the MatrixList
    handles, 1 + 3G + i), StateSet j = packed region j."""
    n = im.drawables.shape[0]
    starts = np.concatenate([[0], np.cumsum(im.state_set_counts)]).astype(np.int64)
    region = np.repeat(np.arange(len(im.state_set_counts)), im.state_set_counts)
    slot_of_pos = (im.drawables["matrix_list_handle"].astype(np.int64) - 1 - 3 * G)
    ss = np.empty(n, np.uint32)
    li = np.empty(n, np.uint32)
    ss[slot_of_pos] = region
    li[slot_of_pos] = np.arange(n) - starts[region]
    pool = np.empty_like(im.drawables)
    pool[slot_of_pos] = im.drawables
    return np.arange(len(im.state_set_counts), dtype=np.uint32), ss, li, pool


@pytest.mark.parametrize("level_n", [3000, 300_000, 5_000_000])
def test_process_from_pool_equals_packed(ctx, level_n):
    """cadr_pack_process_drawables (records read in slot order, outputs
    scattered to their packed positions) equals processDrawables over the
    packed array; extra slots laid out after the drawn positions are not
    touched."""
    G = 4096 if level_n > 3000 else None
    kw = dict(n=level_n, num_state_sets=12, num_geometries=G or min(level_n, 4096))
    probe = tier_a.build(seed=41, base=1 << 40, **kw)
    buf = ctx.alloc(probe.image.nbytes + 4096)
    im = tier_a.build(seed=41, base=buf.ptr, **kw)
    r_ind, r_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables,
                                          threads=bind.max_threads())
    ctx.upload(buf, im.image)
    n = im.drawables.shape[0]
    dfs, ss, li, pool = creation_order_layout(im, kw["num_geometries"])
    # 1,000 more slots in a trailing StateSet that is not drawn (valid
    # records, so that reading them would be harmless but visible).
    extra = 1000
    dfs = np.append(dfs, len(dfs)).astype(np.uint32)
    ss = np.concatenate([ss, np.full(extra, len(dfs) - 1, np.uint32)])
    li = np.concatenate([li, np.arange(extra, dtype=np.uint32)])
    pool = np.concatenate([pool, im.drawables[:extra]])
    pk = lib.Pack(ctx, n + extra)
    pk.set_layout(dfs, ss, li)
    pk.upload(pool)
    ind, ptr = ctx.alloc((n + extra) * 16), ctx.alloc((n + extra) * 32)
    ctx.upload(ind, np.full((n + extra) * 4, 0xDEADBEEF, np.uint32))
    ctx.upload(ptr, np.full((n + extra) * 4, 0xDEADBEEFDEADBEEF, np.uint64))
    pk.process_drawables(im.level, im.root, n, ind, ptr)
    ctx.sync()
    assert ctx.check_device_error() == 0
    g_ind = ctx.download(ind, np.uint32, (n + extra, 4))
    g_ptr = ctx.download(ptr, np.uint64, (n + extra, 4))
    assert np.array_equal(g_ind[:n], r_ind) and np.array_equal(g_ptr[:n], r_ptr)
    assert (g_ind[n:] == 0xDEADBEEF).all() and (g_ptr[n:] == 0xDEADBEEFDEADBEEF).all()
