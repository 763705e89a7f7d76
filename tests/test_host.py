"""Host-side logic: generators, views, Tier A images, multi-rank helpers."""
import numpy as np

from cadr_gb300 import multigpu, rng, scenes, tier_a
from cadr_gb300.views import Camera, OrthoBox, shadow_cascades


def test_counter_rng_is_prefix_stable():
    st = rng.Stream(5, "x")
    a = st.uniform(np.arange(1000, dtype=np.uint64))
    b = st.uniform(np.arange(100, dtype=np.uint64))
    assert np.array_equal(a[:100], b)
    q1 = rng.unit_quaternions(rng.Stream(1, "q"), 500)
    q2 = rng.unit_quaternions(rng.Stream(1, "q"), 50)
    assert np.array_equal(q1[:50], q2)


def test_transforms_are_rigid_with_scale():
    m = scenes.transforms(3, "t", 1000, 20.0, (0.5, 2.0)).astype(np.float64).reshape(-1, 4, 4)
    r = m[:, :3, :3]
    s2 = np.einsum("nij,nij->ni", r, r)  # squared column lengths (column-major rows here)
    assert np.allclose(s2 / s2[:, :1], 1.0, atol=1e-5)
    assert np.all((s2[:, 0] >= 0.25 - 1e-5) & (s2[:, 0] <= 4 + 1e-4))
    assert np.all(np.abs(m[:, 3, :3]) <= 20.0)


def test_config_shapes():
    c1 = scenes.config1()
    assert c1.n == 10_000 and c1.num_state_sets == 8 and c1.level_sizes == [100] and c1.num_lods == 1
    assert np.all(np.diff(c1.state_set_offsets.astype(np.int64)) >= 0)
    assert c1.state_set_offsets[-1] == c1.n
    c2 = scenes.config2(n=1 << 16)
    assert c2.level_sizes == [16, 256, 4096] and c2.num_state_sets == 256 and c2.num_lods == 3
    assert np.all(np.diff(c2.level_parent[2].astype(np.int64)) >= 0)
    counts = np.diff(c2.state_set_offsets.astype(np.int64))
    assert counts[0] > counts[10] > counts[200]  # Zipf
    c3 = scenes.config3(n=1 << 14)
    assert c3.n == 1 << 14 and c3.level_sizes[0] == 1 and len(c3.level_sizes) >= 4
    for l in range(1, len(c3.level_sizes)):
        br = np.bincount(c3.level_parent[l], minlength=c3.level_sizes[l - 1])
        assert br.min() >= 2 and br.max() <= 16


def test_views_have_unit_normals_and_contain_their_axis():
    cam = Camera(np.array([1.0, 2.0, 3.0]), np.array([0.3, -0.2, -1.0]), 50.0, 1.5, 0.5, 1000.0, 1080, (64, 16))
    v = cam.to_view()
    n = v["planes"][0][:, :3].astype(np.float64)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    f = np.array([0.3, -0.2, -1.0]) / np.linalg.norm([0.3, -0.2, -1.0])
    p = np.array([1.0, 2.0, 3.0]) + 10 * f
    assert np.all(v["planes"][0][:, :3] @ p + v["planes"][0][:, 3] > 0)
    casc = shadow_cascades(cam, np.array([0.3, -1.0, 0.2]), 4, 500.0)
    assert len(casc) == 4 and all(isinstance(c, OrthoBox) for c in casc)
    assert casc[0].to_view()["perspective"][0] == 0


def test_config4_views():
    scs = scenes.config4(num_scenes=2, lo=1000, hi=3000)
    assert len(scs) == 2 and all(len(s.views) == 8 for s in scs)
    assert sum(int(v["perspective"][0]) for v in scs[0].views) == 4


def test_tier_a_image_levels():
    for n, extra, lvl in [(200, 0, 1), (3000, 0, 2), (500, 4_200_000, 3)]:
        im = tier_a.build(n, seed=1, base=1 << 40, num_geometries=50, extra_handles=extra)
        assert im.level == lvl
        assert im.drawables.shape == (n,)
        assert int(im.state_set_counts.sum()) == n


def test_shard_helpers():
    off = np.array([0, 3, 3, 10], np.uint32)
    assert multigpu.shard_bounds(10, 3, 2) == (8, 10)
    assert multigpu.local_offsets(off, 4, 8).tolist() == [0, 0, 0, 4]
    ca = np.array([[1, 0, 2], [2, 0, 1]])
    assert multigpu.placement(ca, off, 1).tolist() == [1, 3, 5]
