"""Output buffers shared by file descriptor (cadr_shared_buffer_*): the
plain pass writes its commands into exportable device memory, the exported
descriptor maps the same memory at a second address (as a Vulkan import
would), and what one mapping writes the other reads, bit for bit."""
import os

import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same
from oracle import bind

pytestmark = pytest.mark.gpu


def test_pass_writes_into_shared_buffer_seen_through_imported_fd(ctx):
    sc = scenes.small_scene(seed=9, n=50_000, num_levels=2, num_state_sets=7)
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    shared = lib.SharedBuffer(ctx, sc.n * 20)
    assert shared.nbytes >= sc.n * 20 and shared.ptr
    out.cmds = shared
    ds.cull(np.ascontiguousarray(sc.views[0]), out)
    ctx.sync()
    assert ctx.check_device_error() == 0
    got = out.fetch()
    assert_same(got, bind.cull(sc, sc.views[0]), sc.state_set_offsets)
    fd = shared.export_fd()
    assert fd >= 0
    try:
        alias = lib.SharedBuffer(ctx, fd=fd, import_bytes=shared.nbytes)
    finally:
        os.close(fd)
    assert alias.ptr != shared.ptr and alias.nbytes == shared.nbytes
    a = ctx.download(alias, np.uint8, (sc.n * 20,))
    assert np.array_equal(a, got["cmds"].view(np.uint8).reshape(-1))
    # Writes through the imported mapping reach the exporter's.
    pattern = np.arange(shared.nbytes // 4, dtype=np.uint32)
    ctx.upload(alias, pattern)
    ctx.sync()
    assert np.array_equal(ctx.download(shared, np.uint32, (shared.nbytes // 4,)), pattern)
    alias.close()
    shared.close()


def test_shared_buffer_arguments_are_checked(ctx):
    with pytest.raises(lib.CadrError) as e:
        lib.SharedBuffer(ctx, 0)
    assert e.value.status == lib.INVALID_ARG
    with pytest.raises(lib.CadrError) as e:
        lib.SharedBuffer(ctx, fd=-1, import_bytes=1 << 21)
    assert e.value.status == lib.INVALID_ARG
    shared = lib.SharedBuffer(ctx, 1000)
    fd = shared.export_fd()
    try:
        with pytest.raises(lib.CadrError) as e:  # not the exported size
            lib.SharedBuffer(ctx, fd=fd, import_bytes=shared.nbytes - 1)
        assert e.value.status == lib.INVALID_ARG
    finally:
        os.close(fd)
    shared.close()
