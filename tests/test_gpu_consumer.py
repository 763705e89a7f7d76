"""The vertex-pulling consumer check (cadr_check_draws) against the oracle:
the Tier A draws of an image with real index, vertex and matrix data are
pulled as the consumer vertex shader would, every checksum, count and flag
equal; corrupted handles are flagged without being dereferenced."""
import numpy as np
import pytest

from cadr_gb300 import lib, tier_a
from oracle import bind

pytestmark = pytest.mark.gpu


def perspective_view():
    view = np.eye(4, dtype=np.float32)
    view[3, 2] = -50.0  # camera 50 units back along +z
    f = 1.0 / np.tan(np.radians(30.0))
    near, far = 0.5, 500.0
    return lib.consumer_view(view.reshape(16), p11=f / (16 / 9), p22=f, p33=far / (near - far),
                             p43=near * far / (near - far), p34=-1.0, p44=0.0)


def tier_a_draws(ctx, n, seed, corrupt=None):
    kw = dict(n=n, num_state_sets=6, num_geometries=64, prims_per_geometry=3, geometry_data=True)
    probe = tier_a.build(seed=seed, base=1 << 40, **kw)
    buf = ctx.alloc(probe.image.nbytes + 4096)
    im = tier_a.build(seed=seed, base=buf.ptr, **kw)
    if corrupt:
        corrupt(im)
    # The oracle first: Tier A reads only the tables, PrimitiveSets and
    # MatrixList headers, which stay inside the image.
    r_ind, r_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables)
    ctx.upload(buf, im.image)
    d = ctx.to_device(im.drawables)
    ind, ptr = ctx.alloc(n * 16), ctx.alloc(n * 32)
    ctx.process_drawables(im.level, im.root, d, n, ind, ptr)
    ctx.sync()
    assert np.array_equal(ctx.download(ind, np.uint32, (n, 4)), r_ind)
    assert np.array_equal(ctx.download(ptr, np.uint64, (n, 4)), r_ptr)
    return im, buf, ind, ptr, r_ind, r_ptr


def run_check(ctx, im, buf, ind, ptr, r_ind, r_ptr, n, view):
    out = ctx.alloc(n * 16)
    ctx.check_draws(ind, ptr, n, [(buf.ptr, im.image.nbytes)], view, out)
    ctx.sync()
    got = ctx.download(out, lib.DRAW_CHECK_DTYPE, (n,))
    ref = bind.check_draws([(im.image, im.base)], r_ind, r_ptr, view)
    return got, ref


def test_consumer_check_matches_oracle(ctx):
    n = 20_000
    im, buf, ind, ptr, r_ind, r_ptr = tier_a_draws(ctx, n, seed=21)
    got, ref = run_check(ctx, im, buf, ind, ptr, r_ind, r_ptr, n, perspective_view())
    assert np.array_equal(got, ref)
    assert (got["flags"] == 0).all()
    assert np.array_equal(got["pulled"], r_ind[:, 0] * r_ind[:, 1])
    assert len(np.unique(got["checksum"])) > n // 2


def test_consumer_check_flags_bad_handles(ctx):
    """The index handle of geometry 0 points past the image and the vertex
    handle of geometry 1 two bytes off alignment: the draws of those
    geometries are flagged, the others are not, and nothing outside the
    image is read."""
    n = 8_000

    def corrupt(im):
        tables = im.image[: 8 * 2048].view(np.uint64)  # the first last-level table: handles 0..2047
        assert im.level >= 1
        tables[2] = np.uint64(im.base + im.image.nbytes + (1 << 20))  # index data of geometry 0
        tables[4] += np.uint64(2)                                      # vertex data of geometry 1

    im, buf, ind, ptr, r_ind, r_ptr = tier_a_draws(ctx, n, seed=22, corrupt=corrupt)
    got, ref = run_check(ctx, im, buf, ind, ptr, r_ind, r_ptr, n, perspective_view())
    assert np.array_equal(got, ref)
    vh = im.drawables["vertex_data_handle"]
    g0, g1 = vh == 1, vh == 4
    assert g0.any() and g1.any()
    assert (got["flags"][g0] == lib.DRAW_BAD_INDEX_READ).all() and (got["pulled"][g0] == 0).all()
    assert (got["flags"][g1] == lib.DRAW_BAD_VERTEX_READ).all()
    assert (got["flags"][~(g0 | g1)] == 0).all()
