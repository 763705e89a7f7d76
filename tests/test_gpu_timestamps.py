"""The per-frame GPU timestamps behind the C++ facade's CadR::FrameInfo
(cadr_context_record_timestamp / cadr_context_read_timestamps)."""
import ctypes as C

import numpy as np
import pytest

from cadr_gb300 import lib, scenes

pytestmark = pytest.mark.gpu


def test_timestamps_of_a_frame_are_ordered(ctx):
    """Four timestamps around a pass read back as nanoseconds after the
    first, in order, the pass's interval positive; a frame that recorded
    only three of them, or one overwritten by four later frames, is
    refused."""
    L = ctx.lib
    sc = scenes.small_scene(seed=5, n=200_000, num_levels=2, num_state_sets=16, num_lods=3)
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ns = (C.c_uint64 * 4)()
    frame = 1000
    lib.check(L.cadr_context_record_timestamp(ctx.handle, frame, 0, None))
    lib.check(L.cadr_context_record_timestamp(ctx.handle, frame, 1, None))
    ds.cull(sc.views[0], out)
    lib.check(L.cadr_context_record_timestamp(ctx.handle, frame, 2, None))
    assert L.cadr_context_read_timestamps(ctx.handle, frame, ns) == lib.INVALID_ARG
    lib.check(L.cadr_context_record_timestamp(ctx.handle, frame, 3, None))
    lib.check(L.cadr_context_read_timestamps(ctx.handle, frame, ns))
    t = np.array(list(ns), np.uint64)
    assert t[0] == 0 and t[0] <= t[1] < t[2] <= t[3]
    assert t[2] - t[1] < 1_000_000_000
    # frames 1001..1004 take the ring's four entries; 1000's is overwritten
    for f in range(1001, 1005):
        for k in range(4):
            lib.check(L.cadr_context_record_timestamp(ctx.handle, f, k, None))
    assert L.cadr_context_read_timestamps(ctx.handle, frame, ns) == lib.INVALID_ARG
    lib.check(L.cadr_context_read_timestamps(ctx.handle, 1004, ns))
    assert L.cadr_context_record_timestamp(ctx.handle, frame, 4, None) == lib.INVALID_ARG
    ctx.check_device_error()
