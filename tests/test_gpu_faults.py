"""Failure detection without a GPU fault: a lookback wait that can never
end (the first tile of a view's scan never publishes its status) runs into
its time limit, the batched pass reports CADR_ERR_TIMEOUT and the context
stays usable.  The plain pass has no waits."""
import numpy as np
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same, gpu_cull
from oracle import bind

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [False, True])
def test_lookback_timeout_is_reported_and_recovered(ctx, use_graph):
    sc = scenes.small_scene(seed=5, n=20_000, num_levels=1, num_state_sets=4)
    ds = lib.DeviceScene(ctx, sc)
    ds.propagate(world_spheres=True)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    arr = lib.batch_views([(ds, np.ascontiguousarray(sc.views[0]), out)])
    tune = lib.Tuning(256, 4, 2, 0)  # 1,024-drawable tiles: 20 of them in the view's scan
    ctx.set_spin_limit_ns(20_000_000)  # 20 ms
    ctx.set_fault(lib.FAULT_SKIP_FIRST_TILE_PUBLISH)
    try:
        lib.cull_batched(ctx, arr, tune, use_graph=use_graph)
        st, bits = ctx.device_error_status()
        assert st == lib.TIMEOUT and bits & 0x1
    finally:
        ctx.set_fault(lib.FAULT_NONE)
        ctx.set_spin_limit_ns(1_000_000_000)
    # The same batch, fault cleared (a graph, if used, is captured again).
    lib.cull_batched(ctx, arr, tune, use_graph=use_graph)
    assert ctx.check_device_error() == 0
    res = out.fetch()
    assert_same(res, bind.cull(sc, sc.views[0]), sc.state_set_offsets)
    res, _, _ = gpu_cull(ctx, sc)
    assert_same(res, bind.cull(sc, sc.views[0]), sc.state_set_offsets)
