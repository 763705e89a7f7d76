"""The allocation-free plain pass, cadr_cull_static_scratch.

It serves callers that cannot allocate device memory while they run (device
memory owned and budgeted by the host application, or a frame loop that
cannot stall on the device-wide synchronisation of cudaMalloc/cudaFree).
It must give exactly the results of cadr_cull, call after call, although
every call reuses the same static scratch array.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes
import dataclasses

import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same
from oracle import bind

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


def test_static_scratch_second_scan_chunk(ctx):
    """Past 16,777,216 drawables the tile scan takes its tiles in a second
    chunk (8,192 tiles of 2,048 drawables per chunk) and carries the running
    region count across.  Region boundaries are placed inside that second
    chunk (in its first and third tile, with an empty region between) so
    that the carry, the restart at a region start and the upper part of the
    static tile and plane areas are all used; both entry points must equal
    the oracle, twice in a row."""
    n = (1 << 24) + 3 * 2048 + 777
    chunk = 8192 * 2048
    base = scenes.config2(n=n, num_state_sets=5)
    offsets = np.array([0, 6_000_000, chunk + 700, chunk + 2 * 2048 + 5, chunk + 2 * 2048 + 5, n], np.uint32)
    sc = dataclasses.replace(base, state_set_offsets=offsets)
    ref = bind.cull(sc, sc.views[0], threads=bind.max_threads())
    assert ref["counts"][2] > 0 and ref["counts"][3] == 0 and ref["counts"][4] > 0
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ds.cull(sc.views[0], out)
    ctx.sync()
    ctx.check_device_error()
    assert_same(out.fetch(), ref, sc.state_set_offsets)
    for _ in range(2):
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
