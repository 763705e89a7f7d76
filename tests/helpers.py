"""Helpers of the GPU parity tests."""
import numpy as np

from cadr_gb300 import lib, scenes
from oracle import bind


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def gpu_cull(ctx, sc, view=None, marginal=True, want_world=False):
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets, marginal=marginal)
    ds.cull(sc.views[0] if view is None else view, out)
    ctx.sync()
    ctx.check_device_error()
    res = out.fetch()
    if want_world:
        b = ds.buffers()
        res["world"] = ctx.download(b.world, np.float32, (sc.n, 16))
    return res, ds, out


def assert_same(gpu, ref, offsets, check_marginal=True):
    assert np.array_equal(gpu["counts"], ref["counts"]), (gpu["counts"], ref["counts"])
    g = bind.valid_cmds(gpu["cmds"], gpu["counts"], offsets)
    r = bind.valid_cmds(ref["cmds"], ref["counts"], offsets)
    assert np.array_equal(bits(g), bits(r))
    if check_marginal:
        assert np.array_equal(gpu["marginal"], ref["marginal"])
    if "world" in gpu and "world" in ref:
        assert np.array_equal(bits(gpu["world"]), bits(ref["world"]))


def scene_from_npz(g):
    lods = np.ascontiguousarray(g["lods"]).view(scenes.LOD_DTYPE).reshape(-1)
    view = np.ascontiguousarray(g["view"]).view(scenes.VIEW_DTYPE).reshape(-1)
    return scenes.Scene("small", 11, [g["level0_local"], g["level1_local"]], [None, g["level1_parent"]],
                        g["local"], g["parent"], g["sphere"], g["geometry"], g["offsets"], lods,
                        int(g["num_lods"][0]), [view])



def pack_layout_from_packed(counts, seed):
    """tier_a.slot_layout: a slot layout whose packing is a given grouping."""
    from cadr_gb300 import tier_a
    return tier_a.slot_layout(counts, seed)
