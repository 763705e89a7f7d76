"""Failure detection without a GPU fault: a lookback wait that can never
end (the first tile's status is never published) runs into its time limit,
the pass reports CADR_ERR_TIMEOUT and the context stays usable."""
import pytest

from cadr_gb300 import lib, scenes
from helpers import assert_same, gpu_cull
from oracle import bind

pytestmark = pytest.mark.gpu


def test_lookback_timeout_is_reported_and_recovered(ctx):
    sc = scenes.small_scene(seed=5, n=20_000, num_levels=1, num_state_sets=4)
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ctx.set_spin_limit_ns(20_000_000)  # 20 ms
    ctx.set_fault(lib.FAULT_SKIP_FIRST_TILE_PUBLISH)
    try:
        ds.cull(sc.views[0], out)
        st, bits = ctx.device_error_status()
        assert st == lib.TIMEOUT and bits & 0x1
    finally:
        ctx.set_fault(lib.FAULT_NONE)
        ctx.set_spin_limit_ns(1_000_000_000)
    res, _, _ = gpu_cull(ctx, sc)
    assert_same(res, bind.cull(sc, sc.views[0]), sc.state_set_offsets)
