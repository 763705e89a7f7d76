"""Seeded synthetic scenes of the benchmark configurations.

Five workloads (the drawable-processing pass's benchmark set):

  C1  plain pass, small scene: 10,000 drawables, 8 StateSets, 100 parents
  C2  plain pass, large CAD scene: 16,777,216 drawables, 256 StateSets (Zipf
      s=1.1), hierarchy 4,096 -> 65,536 -> 1,048,576 -> drawables, 3 LODs
  C3  deep hierarchy: 4,194,304 drawables, BFS tree with branching U{2..16},
      16 StateSets, 2 LODs
  C4  batched: 32 scenes (1,000 .. 2,000,000 drawables, log-uniform), 8 views each
  C5  serving: 64 scenes (10,000 .. 8,000,000 drawables, log-uniform)

Frozen generation rules (the workloads have no public dataset; these rules
are the definition):
  * rotations uniform (unit quaternions, rejection from the 4-cube);
    internal-level transforms: translation U[-500,500]^3 (level 0 of C2-style
    scenes: U[-1e4,1e4]^3), isotropic scale U[0.5,2]; drawable (leaf)
    transforms: translation U[-20,20]^3, scale 1;
  * internal levels are in breadth-first order (children of a node are
    contiguous, parents non-decreasing); leaves are generated in hierarchy
    order, assigned a StateSet, then stably grouped by StateSet, which is how
    the reference stores drawables (one contiguous list per StateSet,
    src/CadR/StateSet.h:47);
  * local bounding sphere centre U[-1,1]^3, radius lognormal;
  * a pool of G = min(N, 4096) geometries, drawable -> geometry uniform;
    LOD k of geometry g is {indexCount, firstIndex, vertexOffset} with
    firstIndex/vertexOffset the running sums of index counts and of
    vertex counts (= max(3, indexCount // 3)) over (g, k) in order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import rng
from .views import VIEW_DTYPE, Camera, shadow_cascades

LOD_DTYPE = np.dtype([("index_count", np.uint32), ("first_index", np.uint32),
                      ("vertex_offset", np.int32), ("reserved", np.uint32)])
CMD_DTYPE = np.dtype([("index_count", np.uint32), ("instance_count", np.uint32),
                      ("first_index", np.uint32), ("vertex_offset", np.int32),
                      ("first_instance", np.uint32)])
assert LOD_DTYPE.itemsize == 16 and CMD_DTYPE.itemsize == 20


@dataclass
class Scene:
    name: str
    seed: int
    level_local: list            # [n_l, 16] float32 per internal level
    level_parent: list           # [n_l] uint32 per level (None for level 0)
    local: np.ndarray            # [N, 16] float32
    parent: np.ndarray | None    # [N] uint32 into the last internal level
    sphere: np.ndarray           # [N, 4] float32
    geometry: np.ndarray         # [N] uint32
    state_set_offsets: np.ndarray  # [S+1] uint32
    lods: np.ndarray             # [G * L] LOD_DTYPE
    num_lods: int
    views: list = field(default_factory=list)   # VIEW_DTYPE records

    @property
    def n(self) -> int:
        return int(self.local.shape[0])

    @property
    def num_state_sets(self) -> int:
        return int(self.state_set_offsets.shape[0] - 1)

    @property
    def num_geometries(self) -> int:
        return int(self.lods.shape[0] // self.num_lods)

    @property
    def level_sizes(self) -> list:
        return [int(a.shape[0]) for a in self.level_local]

    def input_bytes(self) -> int:
        b = self.local.nbytes + self.sphere.nbytes + self.geometry.nbytes
        b += self.parent.nbytes if self.parent is not None else 0
        for loc, par in zip(self.level_local, self.level_parent):
            b += loc.nbytes + (par.nbytes if par is not None else 0)
        return b + self.state_set_offsets.nbytes + self.lods.nbytes


# ---------------------------------------------------------------------------

def transforms(seed: int, name: str, n: int, t_range: float, s_range=(1.0, 1.0)) -> np.ndarray:
    """n random TRS matrices (column-major float32 [n, 16])."""
    idx = np.arange(n, dtype=np.uint64)
    q = rng.unit_quaternions(rng.Stream(seed, name + ".rot"), n)
    st = rng.Stream(seed, name + ".trans")
    t = [st.uniform_range(idx * np.uint64(3) + np.uint64(c), -t_range, t_range) for c in range(3)]
    if s_range[0] == s_range[1]:
        s = np.full(n, s_range[0], np.float64)
    else:
        s = rng.Stream(seed, name + ".scale").uniform_range(idx, s_range[0], s_range[1])
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    m = np.zeros((n, 16), np.float32)
    # column 0
    m[:, 0] = (1.0 - 2.0 * (y * y + z * z)) * s
    m[:, 1] = (2.0 * (x * y + w * z)) * s
    m[:, 2] = (2.0 * (x * z - w * y)) * s
    # column 1
    m[:, 4] = (2.0 * (x * y - w * z)) * s
    m[:, 5] = (1.0 - 2.0 * (x * x + z * z)) * s
    m[:, 6] = (2.0 * (y * z + w * x)) * s
    # column 2
    m[:, 8] = (2.0 * (x * z + w * y)) * s
    m[:, 9] = (2.0 * (y * z - w * x)) * s
    m[:, 10] = (1.0 - 2.0 * (x * x + y * y)) * s
    # column 3: translation
    m[:, 12], m[:, 13], m[:, 14] = t
    m[:, 15] = 1.0
    return m


def spheres(seed: int, n: int, mu: float, sigma: float) -> np.ndarray:
    idx = np.arange(n, dtype=np.uint64)
    st = rng.Stream(seed, "sphere.center")
    out = np.empty((n, 4), np.float32)
    for c in range(3):
        out[:, c] = st.uniform_range(idx * np.uint64(3) + np.uint64(c), -1.0, 1.0)
    out[:, 3] = rng.lognormal(rng.Stream(seed, "sphere.radius"), n, mu, sigma)
    return out


def lod_table(index_counts: np.ndarray) -> np.ndarray:
    """index_counts [G, L] -> LOD_DTYPE [G*L] with packed running offsets."""
    ic = np.asarray(index_counts, np.int64).reshape(-1)
    vc = np.maximum(3, ic // 3)
    out = np.zeros(ic.shape[0], LOD_DTYPE)
    out["index_count"] = ic
    out["first_index"] = np.concatenate([[0], np.cumsum(ic)[:-1]])
    out["vertex_offset"] = np.concatenate([[0], np.cumsum(vc)[:-1]])
    return out


def group_by_state_set(ss: np.ndarray, num_state_sets: int):
    """Stable grouping permutation and the region offsets [S+1]."""
    order = np.argsort(ss, kind="stable")
    counts = np.bincount(ss, minlength=num_state_sets)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    return order, offsets


def _assemble(name, seed, level_local, level_parent, leaf_parent, n, num_state_sets, ss,
              radius_mu, radius_sigma, index_counts_fn, num_lods):
    local = transforms(seed, "leaf", n, 20.0)
    sph = spheres(seed, n, radius_mu, radius_sigma)
    G = min(n, 4096)
    geom = rng.Stream(seed, "geometry").integers(np.arange(n, dtype=np.uint64), 0, G - 1)
    order, offsets = group_by_state_set(ss, num_state_sets)
    lods = lod_table(index_counts_fn(G))
    return Scene(
        name=name, seed=seed, level_local=level_local, level_parent=level_parent,
        local=np.ascontiguousarray(local[order]),
        parent=None if leaf_parent is None else np.ascontiguousarray(leaf_parent[order]).astype(np.uint32),
        sphere=np.ascontiguousarray(sph[order]),
        geometry=np.ascontiguousarray(geom[order]).astype(np.uint32),
        state_set_offsets=offsets, lods=lods, num_lods=num_lods)


def _fanout_levels(seed: int, sizes: list, top_range: float):
    """Internal levels of a fan-out hierarchy: level l node i has parent
    i * n_{l-1} // n_l (contiguous children, non-decreasing parents)."""
    level_local, level_parent = [], []
    for l, n in enumerate(sizes):
        level_local.append(transforms(seed, f"level{l}", n, top_range if l == 0 else 500.0, (0.5, 2.0)))
        if l == 0:
            level_parent.append(None)
        else:
            level_parent.append(((np.arange(n, dtype=np.int64) * sizes[l - 1]) // n).astype(np.uint32))
    return level_local, level_parent


def _leaf_parents(n: int, n_parent: int) -> np.ndarray:
    return ((np.arange(n, dtype=np.int64) * n_parent) // n).astype(np.uint32)


# ---------------------------------------------------------------------------
# Cameras.

def _bounds_camera(seed: int, tag: str, half_extent: float, fov_y: float, aspect: float,
                   near: float, far: float, height: int, thresholds) -> Camera:
    """Camera at a random position inside the scene bounds [-h, h]^3, on the
    shell between 60% and 80% of the half extent along its largest axis,
    looking at the scene centre (about 20-40% of a C2 scene is visible)."""
    st = rng.Stream(seed, "camera." + tag)
    u = np.array([st.uniform_range(np.array([i], np.uint64), -1.0, 1.0)[0] for i in range(3)])
    shell = 0.6 + 0.2 * st.uniform(np.array([3], np.uint64))[0]
    p = u / np.abs(u).max() * shell * half_extent
    return Camera(position=p, forward=-p, fov_y_deg=fov_y, aspect=aspect, near=near, far=far,
                  height_px=height, lod_thresholds_px=tuple(thresholds))


# ---------------------------------------------------------------------------
# The configurations.

def config1(seed: int = 0, n: int = 10_000) -> Scene:
    """C1: 10,000 drawables in 8 StateSets (uniform), 100 parents, 1 LOD."""
    n_par = 100
    level_local = [transforms(seed, "level0", n_par, 500.0, (0.5, 2.0))]
    level_parent = [None]
    idx = np.arange(n, dtype=np.uint64)
    leaf_parent = rng.Stream(seed, "leaf.parent").integers(idx, 0, n_par - 1).astype(np.uint32)
    ss = rng.Stream(seed, "stateset").integers(idx, 0, 7)
    sc = _assemble("C1", seed, level_local, level_parent, leaf_parent, n, 8, ss, 0.0, 0.5,
                   lambda G: rng.Stream(seed, "lod.count").integers(
                       np.arange(G, dtype=np.uint64), 36, 3000).reshape(G, 1), 1)
    cam = Camera(position=np.zeros(3), forward=np.array([0.0, 0.0, -1.0]), fov_y_deg=60.0,
                 aspect=16.0 / 9.0, near=0.1, far=2000.0, height_px=1080)
    sc.views = [cam.to_view()]
    return sc


def config2(seed: int = 1, n: int = 16_777_216, num_state_sets: int = 256) -> Scene:
    """C2: the large CAD scene (4-level hierarchy, 256 Zipf StateSets, 3 LODs).
    Smaller n keeps the same rules with level sizes n/16^3, n/16^2, n/16."""
    sizes = [max(1, n >> 12), max(1, n >> 8), max(1, n >> 4)]
    level_local, level_parent = _fanout_levels(seed, sizes, 1e4)
    leaf_parent = _leaf_parents(n, sizes[-1])
    ss = rng.zipf_choice(rng.Stream(seed, "stateset"), n, num_state_sets, 1.1)
    sc = _assemble("C2", seed, level_local, level_parent, leaf_parent, n, num_state_sets, ss,
                   -1.0, 1.0, lambda G: np.tile(np.array([[3000, 600, 120]]), (G, 1)), 3)
    cam = _bounds_camera(seed, "main", 1e4, 45.0, 16.0 / 9.0, 0.5, 5e4, 2160, (64.0, 16.0))
    sc.views = [cam.to_view()]
    return sc


def config3(seed: int = 2, n: int = 4_194_304) -> Scene:
    """C3: deep BFS tree, branching U{2..16} per node, grown level by level
    from one root until the next level would reach n nodes; that level is
    truncated to n nodes, which are the drawables."""
    sizes = [1]
    parents = [None]
    st = rng.Stream(seed, "branching")
    base = 0
    while True:
        nl = sizes[-1]
        b = st.integers(np.arange(base, base + nl, dtype=np.uint64), 2, 16)
        base += nl
        par = np.repeat(np.arange(nl, dtype=np.uint32), b)
        if par.shape[0] >= n:
            leaf_parent = par[:n]
            break
        sizes.append(int(par.shape[0]))
        parents.append(par)
    level_local = [transforms(seed, f"level{l}", s, 0.0 if l == 0 else 500.0, (0.5, 2.0))
                   for l, s in enumerate(sizes)]
    ss = rng.Stream(seed, "stateset").integers(np.arange(n, dtype=np.uint64), 0, 15)
    sc = _assemble("C3", seed, level_local, parents, leaf_parent, n, 16, ss, -2.0, 1.5,
                   lambda G: np.tile(np.array([[3000, 600]]), (G, 1)), 2)
    cam = _bounds_camera(seed, "main", _level_extent(sc), 45.0, 16.0 / 9.0, 0.5, 5e4, 2160,
                         (32.0,))
    sc.views = [cam.to_view()]
    return sc


def world_positions(sc: Scene) -> np.ndarray:
    """Approximate (float64) world positions of the drawables, used only to
    place cameras; the pass itself never sees these numbers."""
    w = None
    for loc, par in zip(sc.level_local, sc.level_parent):
        m = loc.astype(np.float64).reshape(-1, 4, 4).transpose(0, 2, 1)  # row-major
        w = m if par is None else np.einsum("nij,njk->nik", w[par.astype(np.int64)], m)
    leaf_t = np.concatenate([sc.local[:, 12:15].astype(np.float64),
                             np.ones((sc.n, 1))], axis=1)
    if w is None:
        return leaf_t[:, :3]
    return np.einsum("nij,nj->ni", w[sc.parent.astype(np.int64)], leaf_t)[:, :3]


def _level_extent(sc: Scene) -> float:
    """Half extent for camera placement: the 90th percentile of the
    drawables' largest absolute world coordinate."""
    p = world_positions(sc)
    return float(np.percentile(np.abs(p).max(axis=1), 90.0))


def scene_sizes(seed: int, count: int, lo: int, hi: int) -> list:
    st = rng.Stream(seed, "scene.sizes")
    u = st.uniform(np.arange(count, dtype=np.uint64))
    return [int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * x))) for x in u]


def multi_scene_views(seed: int, sc: Scene, tag: str, num_persp: int, num_cascades: int) -> list:
    """Views of one batched/serving scene: num_persp cameras at random
    positions inside the scene bounds with fovY U[30,90], plus num_cascades
    orthographic shadow cascades of the first camera."""
    st = rng.Stream(seed, "views." + tag)
    views = []
    cams = []
    for i in range(num_persp):
        fov = 30.0 + 60.0 * st.uniform(np.array([i], np.uint64))[0]
        cam = _bounds_camera(seed, f"{tag}.{i}", 1e4, fov, 16.0 / 9.0, 0.5, 5e4, 2160,
                             (64.0, 16.0))
        cams.append(cam)
        views.append(cam.to_view())
    if num_cascades:
        light = np.array([0.3, -1.0, 0.2])
        for box in shadow_cascades(cams[0], light, num_cascades, 2e4, (64.0, 16.0)):
            views.append(box.to_view())
    return views


def config4(seed: int = 3, num_scenes: int = 32, lo: int = 1000, hi: int = 2_000_000,
            views_per_scene: int = 8) -> list:
    """C4: scenes built as C2 with per-scene seeds 3000+i; per scene
    views_per_scene views: views_per_scene-4 perspective cameras and the 4
    orthographic shadow cascades of the first camera."""
    out = []
    for i, n in enumerate(scene_sizes(seed, num_scenes, lo, hi)):
        sc = config2(seed=3000 + i, n=n)
        sc.name = f"C4.{i}"
        nc = 4 if views_per_scene >= 5 else 0
        sc.views = multi_scene_views(3000 + i, sc, "c4", views_per_scene - nc, nc)
        out.append(sc)
    return out


def config5_scenes(seed: int = 4, num_scenes: int = 64, lo: int = 10_000,
                   hi: int = 8_000_000) -> list:
    """C5: resident scenes of the serving form, built as C2 (seeds 4000+i)."""
    out = []
    for i, n in enumerate(scene_sizes(seed, num_scenes, lo, hi)):
        sc = config2(seed=4000 + i, n=n)
        sc.name = f"C5.{i}"
        out.append(sc)
    return out


def random_view(seed: int, index: int, fov_lo=30.0, fov_hi=90.0) -> np.ndarray:
    """A serving request's camera (fovY U[30,90]) inside the C2-style bounds."""
    st = rng.Stream(seed, "request.fov")
    fov = fov_lo + (fov_hi - fov_lo) * st.uniform(np.array([index], np.uint64))[0]
    return _bounds_camera(seed, f"req.{index}", 1e4, fov, 16.0 / 9.0, 0.5, 5e4, 2160,
                          (64.0, 16.0)).to_view()


def small_scene(seed: int, n: int, num_levels: int = 2, num_state_sets: int = 5,
                num_lods: int = 3, empty_state_sets: tuple = (), fanout: int = 4,
                camera_extent: float = 600.0) -> Scene:
    """Parity-test scene of arbitrary size: a fan-out hierarchy with
    num_levels internal levels (0 = none), num_state_sets uniform StateSets
    (those in empty_state_sets receive no drawables), num_lods LODs."""
    if num_levels:
        sizes = [max(1, n // fanout ** (num_levels - l)) for l in range(num_levels)]
        level_local, level_parent = _fanout_levels(seed, sizes, 500.0)
        leaf_parent = _leaf_parents(n, sizes[-1])
    else:
        level_local, level_parent, leaf_parent = [], [], None
    live = [s for s in range(num_state_sets) if s not in set(empty_state_sets)]
    pick = rng.Stream(seed, "stateset").integers(np.arange(n, dtype=np.uint64), 0, len(live) - 1)
    ss = np.array(live, np.int64)[pick] if n else np.zeros(0, np.int64)
    counts = [3000, 600, 120, 24][:num_lods]
    sc = _assemble("small", seed, level_local, level_parent, leaf_parent, n, num_state_sets, ss,
                   1.5, 1.0, lambda G: np.tile(np.array([counts]), (G, 1)), num_lods) if n else None
    if sc is None:
        sc = Scene("small", seed, level_local, level_parent, np.zeros((0, 16), np.float32),
                   None if not num_levels else np.zeros(0, np.uint32), np.zeros((0, 4), np.float32),
                   np.zeros(0, np.uint32), np.zeros(num_state_sets + 1, np.uint32),
                   lod_table(np.tile(np.array([counts]), (1, 1))), num_lods)
    cam = _bounds_camera(seed, "small", camera_extent, 60.0, 16.0 / 9.0, 0.5, 5e4, 1080,
                         (48.0, 12.0, 3.0)[:num_lods - 1])
    sc.views = [cam.to_view()]
    return sc


def band_scene(seed: int, n: int) -> Scene:
    """Parity-test scene for the marginal band: n spheres placed against the
    six planes of C1's camera, each at a signed surface distance
    t = dist + r drawn from U[-4e-5, 4e-5] from one plane (computed in
    double, stored as float translations of identity leaf matrices, no
    hierarchy), so that a good share of them lies inside the 1e-5 band and
    the rest just outside it.  Points are taken at depths up to 20 units,
    where a float coordinate still resolves the band."""
    view = config1().views[0]
    planes = view["planes"].reshape(6, 4).astype(np.float64)
    idx = np.arange(n, dtype=np.uint64)
    st = rng.Stream(seed, "band")
    p = st.integers(idx * np.uint64(8), 0, 5)
    depth = 0.2 + 19.8 * st.uniform(idx * np.uint64(8) + np.uint64(1))
    half = math.tan(math.radians(30.0))
    x = st.uniform_range(idx * np.uint64(8) + np.uint64(2), -1.0, 1.0) * depth * half * 16.0 / 9.0
    y = st.uniform_range(idx * np.uint64(8) + np.uint64(3), -1.0, 1.0) * depth * half
    pts = np.stack([x, y, -depth], axis=1)
    nrm, d = planes[p, :3], planes[p, 3]
    on = pts - nrm * ((nrm * pts).sum(axis=1) + d)[:, None]       # projected onto plane p
    r = np.exp(-2.0 + 1.5 * st.uniform(idx * np.uint64(8) + np.uint64(4)))
    t = st.uniform_range(idx * np.uint64(8) + np.uint64(5), -4e-5, 4e-5)
    c = on + nrm * (t - r)[:, None]
    local = np.tile(np.eye(4, dtype=np.float32).reshape(1, 16), (n, 1))
    local[:, 12:15] = c.astype(np.float32)
    sph = np.zeros((n, 4), np.float32)
    sph[:, 3] = r.astype(np.float32)
    ss = st.integers(idx * np.uint64(8) + np.uint64(6), 0, 3)
    order, offsets = group_by_state_set(ss, 4)
    G = 16
    geom = st.integers(idx * np.uint64(8) + np.uint64(7), 0, G - 1).astype(np.uint32)
    sc = Scene("band", seed, [], [], np.ascontiguousarray(local[order]), None,
               np.ascontiguousarray(sph[order]), np.ascontiguousarray(geom[order]), offsets,
               lod_table(np.tile(np.array([[300, 30]]), (G, 1))), 2)
    sc.views = [view]
    return sc

