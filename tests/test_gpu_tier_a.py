"""Tier A (processDrawables) on the GPU against the oracle, at handle-table
depths 1, 2 and 3: every output word must match."""
import json
import os

import numpy as np
import pytest

from cadr_gb300 import lib, tier_a
from oracle import bind

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def run_tier_a(ctx, im_kwargs, seed=7):
    probe = tier_a.build(seed=seed, base=1 << 40, **im_kwargs)
    buf = ctx.alloc(probe.image.nbytes + 4096)
    im = tier_a.build(seed=seed, base=buf.ptr, **im_kwargs)
    # The oracle first: it raises if any lookup would leave the image, so the
    # GPU only ever dereferences addresses inside the uploaded buffer.
    r_ind, r_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables)
    ctx.upload(buf, im.image)
    n = im.drawables.shape[0]
    d = ctx.to_device(im.drawables)
    ind = ctx.alloc(max(16, n * 16))
    ptr = ctx.alloc(max(16, n * 32))
    ctx.process_drawables(im.level, im.root, d, n, ind, ptr)
    ctx.sync()
    g_ind = ctx.download(ind, np.uint32, (n, 4))
    g_ptr = ctx.download(ptr, np.uint64, (n, 4))
    return im, g_ind, g_ptr, r_ind, r_ptr


@pytest.mark.parametrize("name", ["level1", "level2", "level3"])
def test_golden_images(ctx, name):
    e = json.load(open(os.path.join(GOLDEN, "tier_a.json")))["images"][name]
    im, g_ind, g_ptr, r_ind, r_ptr = run_tier_a(ctx, e["kwargs"])
    assert im.level == e["level"]
    assert np.array_equal(g_ind, r_ind)
    assert np.array_equal(g_ptr, r_ptr)


def test_large_level3(ctx):
    im, g_ind, g_ptr, r_ind, r_ptr = run_tier_a(ctx, dict(n=1 << 21, num_geometries=4096, prims_per_geometry=4))
    assert im.level == 3
    assert np.array_equal(g_ind, r_ind)
    assert np.array_equal(g_ptr, r_ptr)


def test_misaligned_and_empty(ctx):
    buf = ctx.alloc(1 << 16)
    assert ctx.lib.cadr_process_drawables(ctx.handle, 1, buf.ptr, buf.ptr + 8, 4, buf.ptr, buf.ptr, None) == lib.INVALID_ARG
    assert ctx.lib.cadr_process_drawables(ctx.handle, 4, buf.ptr, buf.ptr, 4, buf.ptr, buf.ptr, None) == lib.INVALID_ARG
    assert ctx.lib.cadr_process_drawables(ctx.handle, 2, buf.ptr, buf.ptr, 0, buf.ptr, buf.ptr, None) == lib.OK


@pytest.mark.parametrize("kw", [
    dict(n=1),
    dict(n=33, num_geometries=5),
    dict(n=32767, matrices_per_list=3),
    dict(n=32769, with_drawable_data=False),
    dict(n=70001, num_geometries=7, prims_per_geometry=5),
])
def test_ragged_sizes_against_oracle(ctx, kw):
    """Counts that end inside a warp, a CTA or one past the shader's
    32,768-workgroup dispatch row; MatrixLists of several matrices, no
    drawable data (handle 0) and uneven PrimitiveSet counts."""
    im, g_ind, g_ptr, r_ind, r_ptr = run_tier_a(ctx, kw, seed=11)
    assert g_ind.shape[0] == kw["n"]
    assert np.array_equal(g_ind, r_ind)
    assert np.array_equal(g_ptr, r_ptr)
