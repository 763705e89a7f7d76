"""The allocation-free plain pass, cadr_cull_static_scratch.

It serves callers that cannot allocate device memory while they run (device
memory owned and budgeted by the host application, or a frame loop that
cannot stall on the device-wide synchronisation of cudaMalloc/cudaFree).
It must give exactly the results of cadr_cull, call after call, although
every call reuses the same static scratch array.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same

pytestmark = pytest.mark.gpu

MAX_DRAWABLES = 16384 * 2048


def _static_cull(ctx, ds, view, out):
    v = np.ascontiguousarray(view, scenes.VIEW_DTYPE)
    lib.check(ctx.lib.cadr_cull_static_scratch(ds.handle, v.ctypes.data, out.cmds.ptr, out.counts.ptr,
                                               out.marginal.ptr, None))


def test_static_scratch_matches_cull_twice(ctx):
    sc = scenes.config2(n=(1 << 20) + 12345)
    ds = lib.DeviceScene(ctx, sc)
    ref_out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(sc.views[0], ref_out)
    ctx.sync()
    ctx.check_device_error()
    ref = ref_out.fetch()
    for _ in range(2):  # two calls in a row share the static scratch
        out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
        _static_cull(ctx, ds, sc.views[0], out)
        ctx.sync()
        ctx.check_device_error()
        assert_same(out.fetch(), ref, sc.state_set_offsets)


def test_static_scratch_rejects_scenes_beyond_its_maximum(ctx):
    d = lib.SceneDesc()
    d.num_levels = 0
    d.num_state_sets = 1
    d.num_drawables = MAX_DRAWABLES + 1
    d.num_geometries = 1
    d.num_lods = 1
    h = lib.vp()
    lib.check(ctx.lib.cadr_scene_create(ctx.handle, ctypes.byref(d), ctypes.byref(h)))
    try:
        lib.check(ctx.lib.cadr_scene_commit(h.value))
        view = scenes.config1().views[0]
        st = ctx.lib.cadr_cull_static_scratch(h.value, view.ctypes.data, 16, 16, None, None)
        assert st == lib.INVALID_ARG
        assert b"exceed the maximum" in ctx.lib.cadr_last_error()
    finally:
        ctx.lib.cadr_scene_destroy(h.value)
