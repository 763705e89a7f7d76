"""The oracle against the reference's own code, golden fixtures and
hand-derived known answers (CPU only)."""
import hashlib
import json
import os

import numpy as np
import pytest

from cadr_gb300 import scenes, tier_a
from cadr_gb300.views import VIEW_DTYPE, Camera

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_oracle_matches_reference_math_fixture(oracle_lib):
    """Matrix products and sphere transforms of the reference code (GLM,
    CadR::BoundingSphere) stored in ref_math.npz: the oracle must reproduce
    every bit."""
    from oracle import bind
    g = np.load(os.path.join(GOLDEN, "ref_math.npz"))
    for i in range(g["a"].shape[0]):
        assert np.array_equal(bits(bind.mat4_mul(g["a"][i], g["b"][i])), bits(g["prod"][i])), i
        assert np.array_equal(bits(bind.sphere_transform(g["a"][i], g["s"][i])), bits(g["sphere"][i])), i


def test_oracle_matches_reference_math_live(oracle_lib):
    """Same check against the reference shim built from the CADR sources
    (only where they are present, i.e. in the build container)."""
    from oracle import bind
    ref = bind.load_ref()
    if ref is None:
        pytest.skip("reference sources not present: oracle/_ref not built")
    rs = np.random.RandomState(3)
    for _ in range(3000):
        a = (rs.standard_normal(16) * rs.choice([1e-4, 1, 1e5])).astype(np.float32)
        b = (rs.standard_normal(16) * rs.choice([1e-4, 1, 1e5])).astype(np.float32)
        s = (rs.standard_normal(4) * rs.choice([1e-3, 1, 1e4])).astype(np.float32)
        s[3] = abs(s[3])
        r = np.empty(16, np.float32)
        ref.ref_mat4_mul(a.ctypes.data, b.ctypes.data, r.ctypes.data)
        assert np.array_equal(bits(bind.mat4_mul(a, b)), bits(r))
        r4 = np.empty(4, np.float32)
        ref.ref_sphere_transform(a.ctypes.data, s.ctypes.data, r4.ctypes.data)
        assert np.array_equal(bits(bind.sphere_transform(a, s)), bits(r4))


def test_reference_radius_is_double_precision(oracle_lib):
    """BoundingSphere.h:85 takes sqrt() in double; a float-only evaluation
    differs from the reference on a large share of inputs."""
    from oracle import bind
    g = np.load(os.path.join(GOLDEN, "ref_math.npz"))
    differs = 0
    for i in range(g["a"].shape[0]):
        m = g["a"][i]
        l = [np.float32(m[4 * c] * m[4 * c]) + np.float32(m[4 * c + 1] * m[4 * c + 1]) for c in range(3)]
        l = [np.float32(np.float32(l[c]) + np.float32(m[4 * c + 2] * m[4 * c + 2])) for c in range(3)]
        mx = max(l)
        f = np.float32(np.sqrt(np.float32(mx), dtype=np.float32) * g["s"][i][3])
        differs += int(bits(np.array([f]))[0] != bits(g["sphere"][i][3:4])[0])
    assert differs > 0


def test_c1_generator_and_oracle_golden(oracle_lib):
    from oracle import bind
    d = json.load(open(os.path.join(GOLDEN, "c1.json")))
    sc = scenes.config1()
    got = {"level0_local": sha(sc.level_local[0]), "local": sha(sc.local), "parent": sha(sc.parent),
           "sphere": sha(sc.sphere), "geometry": sha(sc.geometry), "offsets": sha(sc.state_set_offsets),
           "lods": sha(sc.lods), "view": sha(sc.views[0])}
    assert got == d["inputs"]
    o = bind.cull(sc, sc.views[0], threads=1, want_world=True)
    assert o["counts"].tolist() == d["outputs"]["counts"]
    assert sha(bind.valid_cmds(o["cmds"], o["counts"], sc.state_set_offsets)) == d["outputs"]["valid_cmds"]
    assert sha(o["marginal"]) == d["outputs"]["marginal"]
    assert sha(o["world"]) == d["outputs"]["world"]
    assert sha(o["world_sphere"]) == d["outputs"]["world_sphere"]


def test_oracle_threads_agree(oracle_lib):
    from oracle import bind
    sc = scenes.config1()
    a = bind.cull(sc, sc.views[0], threads=1, want_world=True)
    b = bind.cull(sc, sc.views[0], threads=4, want_world=True)
    for k in a:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_small_golden(oracle_lib):
    from oracle import bind
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    sc = scenes.small_scene(seed=11, n=1500, num_levels=2, num_state_sets=6, num_lods=3,
                            empty_state_sets=(3,), camera_extent=600.0)
    assert np.array_equal(bits(sc.local), bits(g["local"]))
    o = bind.cull(sc, sc.views[0], threads=2, want_world=True)
    assert np.array_equal(o["counts"], g["counts"])
    assert o["counts"][3] == 0
    v = bind.valid_cmds(o["cmds"], o["counts"], sc.state_set_offsets).view(np.uint32).reshape(-1, 5)
    assert np.array_equal(v, g["valid_cmds"])
    assert np.array_equal(o["marginal"], g["marginal"])
    assert np.array_equal(bits(o["world"]), bits(g["world"]))


def test_tier_a_golden(oracle_lib):
    from oracle import bind
    d = json.load(open(os.path.join(GOLDEN, "tier_a.json")))
    for name, e in d["images"].items():
        im = tier_a.build(seed=d["seed"], base=d["base"], **e["kwargs"])
        assert im.level == e["level"], name
        assert sha(im.image) == e["image"], name
        ind, ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables, threads=2)
        assert sha(ind) == e["indirect"], name
        assert sha(ptr) == e["pointers"], name


# ---------------------------------------------------------------------------
# Known answers derived by hand from processDrawables.comp:77-113.

def _hand_image(level, base=0x100000):
    """A hand-laid memory image at `base`, handle table of `level` levels,
    one PrimitiveSet array and one MatrixList."""
    img = np.zeros(0x40000, np.uint8)
    u64 = img.view(np.uint64)
    u32 = img.view(np.uint32)
    # addresses (byte offsets from base)
    PS, ML = 0x30000, 0x30100
    u32[PS // 4: PS // 4 + 6] = [11, 100, 22, 200, 33, 300]     # 3 PrimitiveSets {count, first}
    u32[ML // 4] = 7                                           # numMatrices
    targets = {5: base + PS, 6: base + ML, 7: 0xAAAA0000, 8: 0xBBBB0000, 9: 0xCCCC0000}
    if level == 1:
        root = base
        for h, a in targets.items():
            u64[h] = a
        hs = {k: k for k in targets}
    elif level == 2:
        # handle h -> table[h >> 11][h & 0x7ff]; use handles in table 1
        root = base + 0x10000
        llt1 = base + 0x8000
        u64[0x10000 // 8 + 0] = base  # table 0 (all zero): handle 0 resolves to 0
        u64[0x10000 // 8 + 1] = llt1
        hs = {}
        for k, a in targets.items():
            h = 2048 + k
            u64[(0x8000 // 8) + (h & 0x7FF)] = a
            hs[k] = h
    else:
        # handle h -> l2[h >> 22] -> l1[(h >> 11) & 0x7ff] -> llt[h & 0x7ff]
        root = base + 0x20000
        l1 = base + 0x18000
        llt = base + 0x8000
        u64[0x20000 // 8 + 0] = base + 0x28000  # routing table 0 -> zero table 0
        u64[0x28000 // 8 + 0] = base
        u64[0x20000 // 8 + 1] = l1
        u64[0x18000 // 8 + 2] = llt
        hs = {}
        for k, a in targets.items():
            h = (1 << 22) + (2 << 11) + k
            u64[0x8000 // 8 + (h & 0x7FF)] = a
            hs[k] = h
    d = np.zeros(2, tier_a.DRAWABLE_DTYPE)
    for i, off in enumerate((0, 16)):
        d[i]["vertex_data_handle"] = hs[7]
        d[i]["index_data_handle"] = hs[8]
        d[i]["matrix_list_handle"] = hs[6]
        d[i]["drawable_data_handle"] = hs[9] if i == 0 else 0
        d[i]["primitive_set_handle"] = hs[5]
        d[i]["primitive_set_offset"] = off
    return img, base, root, d


@pytest.mark.parametrize("level", [1, 2, 3])
def test_tier_a_known_answers(oracle_lib, level):
    from oracle import bind
    img, base, root, d = _hand_image(level)
    ind, ptr = bind.process_drawables(img, base, level, root, d, threads=1)
    assert ind.tolist() == [[11, 7, 100, 0], [33, 7, 300, 0]]
    ml = base + 0x30100
    # handle 0 resolves through entry 0 of the tables, which is 0
    assert ptr.tolist() == [[0xAAAA0000, 0xBBBB0000, ml, 0xCCCC0000], [0xAAAA0000, 0xBBBB0000, ml, 0]]


# ---------------------------------------------------------------------------
# The reference's processDrawables shader itself, compiled as C++ from the
# CADR sources (oracle/ref_shader_shim.h); only where they are present, i.e.
# in the build container.

def _ref_shader():
    from oracle import bind
    if bind.load_ref_shader() is None:
        pytest.skip("reference shader not built (needs the CADR sources)")
    return bind


REF_BASE = 0x7E0000000000


def test_tier_a_reference_shader_golden(oracle_lib):
    """The golden Tier A hashes are the reference shader's outputs."""
    bind = _ref_shader()
    d = json.load(open(os.path.join(GOLDEN, "tier_a.json")))
    for name, e in d["images"].items():
        im = tier_a.build(seed=d["seed"], base=d["base"], **e["kwargs"])
        r = bind.ref_shader_process_drawables(im.image, im.base, im.level, im.root, im.drawables)
        if r is None:
            pytest.skip("address range of the golden images is taken in this process")
        assert sha(r[0]) == e["indirect"], name
        assert sha(r[1]) == e["pointers"], name


@pytest.mark.parametrize("level", [1, 2, 3])
def test_tier_a_reference_shader_known_answers(oracle_lib, level):
    bind = _ref_shader()
    img, base, root, d = _hand_image(level, base=REF_BASE)
    r = bind.ref_shader_process_drawables(img, base, level, root, d)
    if r is None:
        pytest.skip("address range taken in this process")
    ind, ptr = r
    assert ind.tolist() == [[11, 7, 100, 0], [33, 7, 300, 0]]
    ml = base + 0x30100
    assert ptr.tolist() == [[0xAAAA0000, 0xBBBB0000, ml, 0xCCCC0000], [0xAAAA0000, 0xBBBB0000, ml, 0]]


@pytest.mark.parametrize("kw", [
    dict(n=1, num_geometries=1),
    dict(n=777, prims_per_geometry=7, matrices_per_list=3),
    dict(n=2500, with_drawable_data=False),
    dict(n=1200, num_geometries=40, geometry_data=True),
    dict(n=900, num_geometries=30, extra_handles=2048 * 2048),
    dict(n=32769, num_geometries=7, prims_per_geometry=5),  # a second dispatch row
])
def test_tier_a_oracle_matches_reference_shader(oracle_lib, kw):
    """The oracle against the reference shader on images of each handle-table
    depth, with several PrimitiveSet counts, MatrixList sizes and without
    drawable data (handle 0)."""
    bind = _ref_shader()
    im = tier_a.build(seed=31, base=REF_BASE, **kw)
    r = bind.ref_shader_process_drawables(im.image, im.base, im.level, im.root, im.drawables)
    if r is None:
        pytest.skip("address range taken in this process")
    o = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables, threads=2)
    assert np.array_equal(o[0], r[0])
    assert np.array_equal(o[1], r[1])


def test_tier_a_out_of_image_is_reported(oracle_lib):
    from oracle import bind
    img, base, root, d = _hand_image(1)
    d[0]["matrix_list_handle"] = 9  # resolves to 0xCCCC0000, outside the image
    with pytest.raises(ValueError):
        bind.process_drawables(img, base, 1, root, d, threads=1)


def test_handle_level_growth():
    # HandleTable.cpp: createHandle1 upgrades at 2047, createHandle2 at 2048^2 - 1
    assert tier_a.handle_level(2047) == 1
    assert tier_a.handle_level(2048) == 2
    assert tier_a.handle_level(2048 * 2048 - 1) == 2
    assert tier_a.handle_level(2048 * 2048) == 3


# ---------------------------------------------------------------------------
# Tier B known answers on hand-placed spheres.

def _one_view():
    cam = Camera(position=np.zeros(3), forward=np.array([0.0, 0.0, -1.0]), fov_y_deg=90.0, aspect=1.0,
                 near=1.0, far=100.0, height_px=1000, lod_thresholds_px=(100.0, 10.0))
    return cam.to_view()


def _hand_scene(centres, radii, ss_of, num_state_sets, num_lods=3):
    n = len(centres)
    local = np.tile(np.eye(4, dtype=np.float32).reshape(1, 16), (n, 1))
    local[:, 12:15] = np.asarray(centres, np.float32)
    sph = np.zeros((n, 4), np.float32)
    sph[:, 3] = radii
    ss = np.asarray(ss_of)
    assert np.all(np.diff(ss) >= 0)
    offsets = np.concatenate([[0], np.cumsum(np.bincount(ss, minlength=num_state_sets))]).astype(np.uint32)
    lods = scenes.lod_table(np.array([[300, 30, 3][:num_lods], [600, 60, 6][:num_lods]]))
    return scenes.Scene("hand", 0, [], [], local, None, sph, (np.arange(n) % 2).astype(np.uint32),
                        offsets, lods, num_lods, [_one_view()])


def test_cull_known_answers(oracle_lib):
    """Spheres in front of, behind and straddling the frustum of a 90 degree
    camera; LOD from projected radius r*500/z against 100 and 10 px."""
    from oracle import bind
    centres = [(0, 0, -10),    # inside, r=3: 3*500/10 = 150 px -> LOD0
               (0, 0, 10),     # behind the camera -> culled
               (0, 0, -50),    # inside, r=1: 10 px -> LOD1 (>= 10)
               (60, 0, -50),   # right of the frustum (x <= z): outside unless r >= 10/sqrt2
               (0, 0, -200),   # beyond far (100) by 100 -> culled
               (0, 0, -99),    # inside, r=0.1: 0.5 px -> LOD2
               (11, 0, -10)]   # outside right plane by 1/sqrt(2) with r=1 -> visible (straddles)
    radii = [3, 1, 1, 1, 1, 0.1, 1]
    ss = [0, 0, 1, 1, 2, 2, 2]
    sc = _hand_scene(centres, radii, ss, 4)
    o = bind.cull(sc, sc.views[0], threads=1)
    assert o["counts"].tolist() == [1, 1, 2, 0]
    v = bind.valid_cmds(o["cmds"], o["counts"], sc.state_set_offsets)
    # (index_count, first_instance): geometry = i % 2 with LODs 300/30/3 and 600/60/6
    got = [(int(c["index_count"]), int(c["first_instance"])) for c in v]
    assert got == [(300, 0), (30, 2), (6, 5), (30, 6)]
    assert all(int(c["instance_count"]) == 1 for c in v)


def test_marginal_band(oracle_lib):
    """The marginal band is absolute: a sphere is marginal when its surface
    lies within 1e-5 of a plane, |dist + r| <= 1e-5, whatever the plane's
    offset.  Near plane at z = -1 (the camera looks down -Z), far plane at
    z = -100."""
    from oracle import bind
    centres = [(0, 0, -0.5),         # touches the near plane: dist + r == 0
               (0, 0, -5),           # well inside
               (0, 0, -0.500005),    # 5e-6 inside the near-plane band
               (0, 0, -0.50003),     # 3e-5 from the near plane: outside the band
               (0, 0, -101.0005)]    # 5e-4 beyond the far plane: outside the band
    sc = _hand_scene(centres, [0.5, 0.5, 0.5, 0.5, 1.0], [0] * 5, 1)
    o = bind.cull(sc, sc.views[0], threads=1)
    m = int(o["marginal"][0])
    assert [(m >> k) & 1 for k in range(5)] == [1, 0, 1, 0, 0]
    # Visibility is the plane test alone: the last sphere is culled.
    assert o["counts"].tolist() == [4]


def test_band_scene_marks_spheres_within_the_band(oracle_lib):
    """On spheres placed against the planes, the oracle's marginal bits are
    the spheres whose surface is within 1e-5 of a plane: recomputed here in
    double, every marked sphere is within the band up to float rounding
    (2e-6 at these depths), and about a quarter of them are marked."""
    from oracle import bind
    sc = scenes.band_scene(seed=5, n=20_000)
    o = bind.cull(sc, sc.views[0], threads=1)
    marked = np.unpackbits(o["marginal"].view(np.uint8), bitorder="little")[:sc.n].astype(bool)
    planes = sc.views[0]["planes"].reshape(6, 4).astype(np.float64)
    c = sc.local[:, 12:15].astype(np.float64)
    t = c @ planes[:, :3].T + planes[:, 3] + sc.sphere[:, 3:4].astype(np.float64)
    near = np.abs(t).min(axis=1)
    assert 0.15 * sc.n < marked.sum() < 0.35 * sc.n
    assert near[marked].max() <= 1e-5 + 2e-6
    assert near[~marked].min() >= 1e-5 - 2e-6


def test_oracle_rejects_bad_offsets(oracle_lib):
    from oracle import bind
    sc = _hand_scene([(0, 0, -5)] * 3, [1, 1, 1], [0, 0, 1], 2)
    sc.state_set_offsets = np.array([0, 2, 1], np.uint32)
    with pytest.raises(ValueError):
        bind.cull(sc, sc.views[0])


def test_view_record_layout():
    v = _one_view()
    assert v.dtype == VIEW_DTYPE and v.nbytes == 144
    # inward normals: the camera-space point (0,0,-10) is inside every plane
    for p in v["planes"][0]:
        assert p[2] * -10.0 + p[3] >= 0


class _StateSet:
    """The reference StateSet as far as packing goes: a drawable list
    (appended on creation, swap-removed on deletion) and child StateSets."""

    def __init__(self):
        self.drawables = []
        self.children = []


def _record_to_command_buffer(ss, out, regions, counter):
    """StateSet::recordToCommandBuffer (StateSet.cpp:198-268): this
    StateSet's list at drawableCounter, then the children depth-first."""
    regions.append((ss, counter))
    n = len(ss.drawables)
    if n:
        out[counter:counter + n] = ss.drawables
        counter += n
    for c in ss.children:
        counter = _record_to_command_buffer(c, out, regions, counter)
    return counter


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_pack_state_sets_matches_recursive_recording(seed):
    """The oracle's packing equals the reference's recursive recording over
    a random StateSet tree whose lists were built by appends and
    swap-removes (so list order is not creation order)."""
    from oracle import bind
    rs = np.random.default_rng(seed)
    S = int(rs.integers(1, 40))
    sets = [_StateSet() for _ in range(S)]
    for i in range(1, S):
        sets[int(rs.integers(0, i))].children.append(sets[i])
    live = {}
    for rec in range(int(rs.integers(0, 3000))):
        s = int(rs.integers(0, S))
        if rs.random() < 0.3 and sets[s].drawables:
            lst = sets[s].drawables
            j = int(rs.integers(0, len(lst)))
            lst[j] = lst[-1]
            lst.pop()
        else:
            sets[s].drawables.append(rec)
    slots = [(s, li, rec) for s in range(S) for li, rec in enumerate(sets[s].drawables)]
    rs.shuffle(slots)
    n = len(slots)
    pool = np.zeros(n, tier_a.DRAWABLE_DTYPE)
    pool["vertex_data_handle"] = [rec for _, _, rec in slots]
    pool["primitive_set_offset"] = [li for _, li, _ in slots]
    # Depth-first order of the tree and the expected packing.
    expect_ids = np.zeros(n, np.int64)
    regions = []
    total = _record_to_command_buffer(sets[0], expect_ids, regions, 0)
    assert total == n
    index = {id(ss): k for k, ss in enumerate(sets)}
    dfs = np.array([index[id(ss)] for ss, _ in regions], np.uint32)
    packed, offsets = bind.pack_state_sets(dfs, [s for s, _, _ in slots], [li for _, li, _ in slots], pool)
    assert np.array_equal(packed["vertex_data_handle"], expect_ids.astype(np.uint64))
    assert offsets[:-1].tolist() == [c for _, c in regions] and offsets[-1] == n


def test_pack_state_sets_rejects_bad_layouts():
    from oracle import bind
    pool = np.zeros(3, tier_a.DRAWABLE_DTYPE)
    with pytest.raises(ValueError):
        bind.pack_state_sets([0, 1], [0, 0, 1], [0, 0, 0], pool)   # list index used twice
    with pytest.raises(ValueError):
        bind.pack_state_sets([0, 1], [0, 0, 2], [0, 1, 0], pool)   # StateSet out of range
    with pytest.raises(ValueError):
        bind.pack_state_sets([0, 0], [0, 0, 1], [0, 1, 0], pool)   # not a permutation
    with pytest.raises(ValueError):
        bind.pack_state_sets([0, 1], [0, 0, 1], [0, 2, 0], pool)   # index past the list


def _mix64(z):
    M = (1 << 64) - 1
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def _consumer_image():
    """One MatrixList (header + 1 matrix), an index buffer and 3 vertices
    at device address B."""
    B = 1 << 32
    img = np.zeros(1024, np.uint8)
    img[0:4] = np.array([1], np.uint32).view(np.uint8)             # numMatrices
    M = np.eye(4, dtype=np.float32)
    M[3, 0:3] = [1.0, 2.0, 3.0]                                    # column 3: translation
    M[0, 0] = 2.0
    img[64:128] = M.reshape(16).view(np.uint8)
    img[256:268] = np.array([2, 0, 1], np.uint32).view(np.uint8)
    pos = np.array([[0.5, -1.0, 0.25], [1.5, 0.75, -2.0], [-0.125, 3.0, 1.0]], np.float32)
    img[512:548] = pos.reshape(9).view(np.uint8)
    ind = np.array([[3, 1, 0, 0]], np.uint32)
    ptr = np.array([[B + 512, B + 256, B, 0]], np.uint64)
    return B, img, ind, ptr, M, pos


def test_consumer_check_known_answer():
    """The oracle's consumer check on a hand-built draw equals the shader
    arithmetic (shader.vert:100-120) done here step by step in float32."""
    from cadr_gb300 import lib
    from oracle import bind
    B, img, ind, ptr, M, pos = _consumer_image()
    view = np.eye(4, dtype=np.float32)
    view[3, 2] = -10.0
    p = dict(p11=1.5, p22=2.0, p33=-1.0, p43=-0.2, p31=0.0, p32=0.0, p34=-1.0, p41=0.0, p42=0.0, p44=0.0)
    v = lib.consumer_view(view.reshape(16), **p)
    out = bind.check_draws([(img, B)], ind, ptr, v)
    f = np.float32

    def col(a, b):  # ((a0 b.x + a1 b.y) + a2 b.z) + a3 b.w, rounded each step
        return np.array([f(f(f(f(a[0][c] * b[0]) + f(a[1][c] * b[1])) + f(a[2][c] * b[2])) + f(a[3][c] * b[3]))
                         for c in range(4)], np.float32)
    W = [col(view, M[c]) for c in range(4)]
    K = 0x9E3779B97F4A7C15
    bits = lambda x: int(np.float32(x).view(np.uint32))
    total = 0
    for k in range(3):
        index = int(np.frombuffer(img[256:268].tobytes(), np.uint32)[k])
        e = col(W, np.array([*pos[index], 1.0], np.float32))
        gx = f(f(f(p["p11"]) * e[0]) + f(f(p["p31"]) * e[2])) + f(f(p["p41"]) * e[3])
        gy = f(f(f(p["p22"]) * e[1]) + f(f(p["p32"]) * e[2])) + f(f(p["p42"]) * e[3])
        gz = f(f(p["p33"]) * e[2]) + f(f(p["p43"]) * e[3])
        gw = f(f(p["p34"]) * e[2]) + f(f(p["p44"]) * e[3])
        ex, ey, ez = f(e[0] / e[3]), f(e[1] / e[3]), f(e[2] / e[3])
        h = (_mix64(bits(gx) | bits(gy) << 32) ^ _mix64((bits(gz) | bits(gw) << 32) ^ K)
             ^ _mix64((bits(ex) | bits(ey) << 32) ^ (2 * K % (1 << 64)))
             ^ _mix64((bits(ez) | index << 32) ^ (3 * K % (1 << 64))))
        total = (total + h) % (1 << 64)
    assert int(out["checksum"][0]) == total and out["pulled"][0] == 3 and out["flags"][0] == 0


@pytest.mark.parametrize("case,flag", [("index outside", 0x1), ("vertex misaligned", 0x2), ("list outside", 0x4),
                                       ("instance past list", 0x8), ("drawable data misaligned", 0x10)])
def test_consumer_check_flags(case, flag):
    from cadr_gb300 import lib
    from oracle import bind
    B, img, ind, ptr, _, _ = _consumer_image()
    ind, ptr = ind.copy(), ptr.copy()
    if case == "index outside":
        ptr[0, 1] = B + 4096
    elif case == "vertex misaligned":
        ptr[0, 0] = B + 514
    elif case == "list outside":
        ptr[0, 2] = B + 8192
    elif case == "instance past list":
        ind[0, 1] = 2
    else:
        ptr[0, 3] = B + 8
    v = lib.consumer_view(np.eye(4, dtype=np.float32).reshape(16), 1.0, 1.0, -1.0, -0.2)
    out = bind.check_draws([(img, B)], ind, ptr, v)
    assert out["flags"][0] == flag
