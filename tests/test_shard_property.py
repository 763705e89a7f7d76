"""The sharded pass's placement rule as a property (CPU, oracle): for
random scenes, StateSet layouts (empty regions included) and rank counts,
culling every contiguous shard on its own and placing its commands at

    offsets[s] + sum over earlier ranks of their count in s

gives the single-rank pass: the same counts and every region's commands in
the same order, firstInstance offset by the shard's first drawable."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from cadr_gb300 import multigpu, scenes  # noqa: E402


@settings(max_examples=60, deadline=None)
@given(n=st.integers(1, 3000), S=st.integers(1, 40), world=st.integers(1, 6), seed=st.integers(0, 10_000),
       levels=st.integers(0, 3), empty_frac=st.floats(0.0, 0.5))
def test_shard_placement_merges_to_the_single_rank_pass(oracle_lib, n, S, world, seed, levels, empty_frac):
    from oracle import bind
    rs = np.random.default_rng(seed)
    empty = tuple(int(s) for s in np.flatnonzero(rs.random(S) < empty_frac))
    if len(empty) == S:
        empty = empty[1:]
    sc = scenes.small_scene(seed=seed, n=n, num_levels=levels, num_state_sets=S, num_lods=3,
                            empty_state_sets=empty, fanout=3)
    ref = bind.cull(sc, sc.views[0], threads=1)
    shards = [multigpu.shard_bounds(n, world, r) for r in range(world)]
    outs = []
    for lo, hi in shards:
        sub = multigpu.shard_scene(sc, lo, hi)
        outs.append((lo, sub, bind.cull(sub, sub.views[0], threads=1) if hi > lo else None))
    counts_all = np.stack([o["counts"] if o is not None else np.zeros(S, np.uint32) for _, _, o in outs])
    assert np.array_equal(counts_all.sum(axis=0), ref["counts"])
    merged = np.zeros_like(ref["cmds"])
    filled = np.zeros(n, bool)
    for rank, (lo, sub, o) in enumerate(outs):
        if o is None:
            continue
        dst = multigpu.placement(counts_all.astype(np.int64), sc.state_set_offsets, rank)
        for s in range(S):
            c = int(o["counts"][s])
            if c == 0:
                continue
            src = int(sub.state_set_offsets[s])
            block = o["cmds"][src:src + c].copy()
            block["first_instance"] += lo
            d = int(dst[s])
            assert not filled[d:d + c].any()
            merged[d:d + c] = block
            filled[d:d + c] = True
    g = bind.valid_cmds(merged, ref["counts"], sc.state_set_offsets)
    r = bind.valid_cmds(ref["cmds"], ref["counts"], sc.state_set_offsets)
    assert np.array_equal(g.view(np.uint8), r.view(np.uint8))
