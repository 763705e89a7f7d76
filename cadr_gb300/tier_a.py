"""Synthetic CadR device-memory images for the Tier A pass.

An image is the bytes of one device buffer at a known base address holding
everything the processDrawables pass dereferences:
  * the handle table, laid out exactly as src/CadR/HandleTable.cpp grows it:
    handles start at 1 (0 is invalid), 2048 entries per table, one level up
    to handle 2047, two levels up to 2048^2 - 1, three beyond
    (createHandle1..3, HandleTable.cpp:142-337);
  * PrimitiveSet arrays {uint32 count, uint32 first} (PrimitiveSet.h:12-15),
    one array per Geometry;
  * MatrixList allocations: a 64-byte header {numMatrices, capacity, 0...}
    followed by the matrices (MatrixList.h:54-59).
Vertex, index and drawable-data allocations are only resolved by the pass,
never read, so their addresses point into a second region that the image
does not hold; with geometry_data=True the image holds them too (vertex
positions, index buffers, MatrixList matrices), for the consumer check.

Drawables are packed in the StateSet depth-first order of
StateSet::recordToCommandBuffer (StateSet.cpp:198-262): a root StateSet with
`num_state_sets` children, drawables grouped by child in child order.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import rng

DRAWABLE_DTYPE = np.dtype([("vertex_data_handle", np.uint64), ("index_data_handle", np.uint64),
                           ("matrix_list_handle", np.uint64), ("drawable_data_handle", np.uint64),
                           ("primitive_set_handle", np.uint64), ("primitive_set_offset", np.uint32),
                           ("padding", np.uint32)])
assert DRAWABLE_DTYPE.itemsize == 48

TABLE = 2048


def handle_level(highest_handle: int) -> int:
    """Table depth after creating handles 1..highest_handle (HandleTable.cpp)."""
    if highest_handle <= TABLE - 1:
        return 1
    if highest_handle <= TABLE * TABLE - 1:
        return 2
    return 3


@dataclass
class TierAImage:
    image: np.ndarray          # uint8, device bytes at `base`
    base: int
    level: int
    root: int                  # device address of the root table
    drawables: np.ndarray      # DRAWABLE_DTYPE [N], StateSet DFS order
    state_set_counts: np.ndarray  # drawables per StateSet (DFS order of the regions)
    num_handles: int


# Consumer data per geometry (geometry_data=True): VERTICES positions of
# 12 bytes and an index buffer of at most prims_per_geometry * 3000 indices.
VERTICES = 1024


def _geometry_bytes(prims_per_geometry):
    return (VERTICES * 12 + prims_per_geometry * 3000 * 4 + 255) & ~255


def _layout(n, G, prims_per_geometry, with_drawable_data, matrices_per_list, extra_handles, geometry_data=False):
    """Handle count, table depth and region sizes of an image."""
    H = 3 * G + n + (n if with_drawable_data else 0) + extra_handles
    level = handle_level(H)
    n_llt = H // TABLE + 1                      # last-level tables
    n_rt = 0 if level < 3 else (H >> 22) + 1    # level-1 routing tables (level 3 only)
    n_tables = n_llt + (1 if level == 2 else 0) + (n_rt + 1 if level == 3 else 0)
    tables_bytes = n_tables * TABLE * 8
    prims_bytes = G * prims_per_geometry * 8
    ml_stride = 64 + 64 * matrices_per_list
    ml_off = (tables_bytes + prims_bytes + 255) & ~255
    size = ml_off + n * ml_stride
    if geometry_data:
        size += G * _geometry_bytes(prims_per_geometry) + n * 64  # geometry, then drawable data
    return H, level, n_llt, n_rt, n_tables, tables_bytes, prims_bytes, ml_stride, ml_off, size


def image_size(n: int, num_geometries: int | None = None, prims_per_geometry: int = 3,
               with_drawable_data: bool = True, matrices_per_list: int = 1, extra_handles: int = 0,
               geometry_data: bool = False) -> int:
    """Bytes of the image build() makes for the same arguments."""
    G = num_geometries or max(1, min(n, 4096))
    return _layout(n, G, prims_per_geometry, with_drawable_data, matrices_per_list, extra_handles, geometry_data)[-1]


def build(n: int, seed: int, base: int, num_state_sets: int = 8, num_geometries: int | None = None,
          prims_per_geometry: int = 3, with_drawable_data: bool = True,
          matrices_per_list: int = 1, extra_handles: int = 0, geometry_data: bool = False) -> TierAImage:
    """Builds the image of n drawables.  base must be 256-byte aligned; it is
    the device address the image will be uploaded to.  With geometry_data
    the vertex, index and drawable-data allocations lie inside the image:
    per geometry VERTICES positions and an index buffer holding its
    PrimitiveSets one after the other (PrimitiveSet.first counted within the
    geometry), and the MatrixList matrices are filled."""
    assert base % 256 == 0
    G = num_geometries or max(1, min(n, 4096))
    idx = np.arange(max(n, 1), dtype=np.uint64)[:n]
    # Handle creation order: per geometry (vertex, index, primitiveSets),
    # then one MatrixList per drawable, then one drawable-data allocation
    # per drawable, then `extra_handles` unused handles.
    h_vertex = 1 + 3 * np.arange(G, dtype=np.uint64)
    h_index = h_vertex + 1
    h_prims = h_vertex + 2
    h_ml = 1 + 3 * G + np.arange(n, dtype=np.uint64)
    h_dd = (1 + 3 * G + n + np.arange(n, dtype=np.uint64)) if with_drawable_data else np.zeros(n, np.uint64)
    H, level, n_llt, n_rt, n_tables, tables_bytes, prims_bytes, ml_stride, ml_off, size = _layout(
        n, G, prims_per_geometry, with_drawable_data, matrices_per_list, extra_handles, geometry_data)
    prims_off = tables_bytes
    img = np.zeros(size, np.uint8)
    tables = img[:tables_bytes].view(np.uint64).reshape(n_tables, TABLE)

    # Addresses of every handle's target.
    addr = np.zeros(H + 1, np.uint64)
    far = np.uint64(base + ((size + (1 << 20)) & ~((1 << 20) - 1)))  # unbacked region
    geo_off = ml_off + n * ml_stride
    gb = _geometry_bytes(prims_per_geometry)
    if geometry_data:
        g_base = np.uint64(base + geo_off) + np.arange(G, dtype=np.uint64) * np.uint64(gb)
        addr[h_vertex.astype(np.int64)] = g_base
        addr[h_index.astype(np.int64)] = g_base + np.uint64(VERTICES * 12)
    else:
        addr[h_vertex.astype(np.int64)] = far + np.arange(G, dtype=np.uint64) * np.uint64(1 << 16)
        addr[h_index.astype(np.int64)] = far + np.uint64(G << 16) + np.arange(G, dtype=np.uint64) * np.uint64(1 << 16)
    addr[h_prims.astype(np.int64)] = np.uint64(base + prims_off) + np.arange(G, dtype=np.uint64) * np.uint64(prims_per_geometry * 8)
    addr[h_ml.astype(np.int64)] = np.uint64(base + ml_off) + idx * np.uint64(ml_stride)
    if with_drawable_data:
        if geometry_data:
            addr[h_dd.astype(np.int64)] = np.uint64(base + geo_off + G * gb) + idx * np.uint64(64)
        else:
            addr[h_dd.astype(np.int64)] = far + np.uint64(2 * G << 16) + idx * np.uint64(256)

    # Last-level tables: llt k holds handles [k*2048, k*2048 + 2047].
    llt = tables[:n_llt].reshape(-1)
    llt[: H + 1] = addr
    llt_addr = np.uint64(base) + np.arange(n_llt, dtype=np.uint64) * np.uint64(TABLE * 8)
    if level == 1:
        root = base
    elif level == 2:
        rt = tables[n_llt]
        rt[:n_llt] = llt_addr
        root = base + n_llt * TABLE * 8
    else:
        # Routing tables m (handles with h >> 22 == m), then the level-2 root.
        for m in range(n_rt):
            lo, hi = m * TABLE, min((m + 1) * TABLE, n_llt)
            tables[n_llt + m, : hi - lo] = llt_addr[lo:hi]
        rt_addr = np.uint64(base) + (n_llt + np.arange(n_rt, dtype=np.uint64)) * np.uint64(TABLE * 8)
        tables[n_llt + n_rt, :n_rt] = rt_addr
        root = base + (n_llt + n_rt) * TABLE * 8

    # PrimitiveSets and MatrixList headers.
    ps = img[prims_off:prims_off + prims_bytes].view(np.uint32).reshape(G, prims_per_geometry, 2)
    st = rng.Stream(seed, "tierA.prims")
    cnt = st.integers(np.arange(G * prims_per_geometry, dtype=np.uint64), 36, 3000).reshape(G, prims_per_geometry)
    ps[:, :, 0] = cnt
    if geometry_data:
        ps[:, :, 1] = np.cumsum(cnt, axis=1) - cnt
    else:
        ps[:, :, 1] = np.cumsum(cnt.reshape(-1)).reshape(G, prims_per_geometry) - cnt
    mlh = img[ml_off:ml_off + n * ml_stride].view(np.uint32).reshape(n, ml_stride // 4)
    mlh[:, 0] = matrices_per_list
    mlh[:, 1] = matrices_per_list
    if geometry_data:
        # Matrices: seeded affine transforms; positions in [-1, 1]^3;
        # indices uniform over the geometry's vertices.
        mats = img[ml_off:ml_off + n * ml_stride].view(np.float32).reshape(n, ml_stride // 4)[:, 16:]
        m = rng.Stream(seed, "tierA.matrices").uniform_range(
            np.arange(n * matrices_per_list * 16, dtype=np.uint64), -1.0, 1.0).astype(np.float32)
        m = m.reshape(n * matrices_per_list, 4, 4)
        m[:, 0:3, 3] = 0.0
        m[:, 3, 3] = 1.0
        m[:, 3, 0:3] *= 100.0
        mats[...] = m.reshape(n, matrices_per_list * 16)
        geo = img[geo_off:geo_off + G * gb].reshape(G, gb)
        pos = rng.Stream(seed, "tierA.positions").uniform_range(
            np.arange(G * VERTICES * 3, dtype=np.uint64), -1.0, 1.0).astype(np.float32)
        geo[:, :VERTICES * 12] = pos.view(np.uint8).reshape(G, VERTICES * 12)
        ni = prims_per_geometry * 3000
        ind = rng.Stream(seed, "tierA.indices").integers(np.arange(G * ni, dtype=np.uint64), 0, VERTICES - 1)
        geo[:, VERTICES * 12:VERTICES * 12 + ni * 4] = ind.astype(np.uint32).view(np.uint8).reshape(G, ni * 4)

    # Drawable records, grouped by StateSet (DFS order of the children).
    g_of = rng.Stream(seed, "tierA.geometry").integers(idx, 0, G - 1)
    p_of = rng.Stream(seed, "tierA.prim").integers(idx, 0, prims_per_geometry - 1)
    ss = rng.Stream(seed, "tierA.stateset").integers(idx, 0, num_state_sets - 1)
    order = np.argsort(ss, kind="stable")
    d = np.zeros(n, DRAWABLE_DTYPE)
    d["vertex_data_handle"] = h_vertex[g_of]
    d["index_data_handle"] = h_index[g_of]
    d["matrix_list_handle"] = h_ml
    d["drawable_data_handle"] = h_dd
    d["primitive_set_handle"] = h_prims[g_of]
    d["primitive_set_offset"] = (p_of * 8).astype(np.uint32)
    d = d[order]
    counts = np.bincount(ss, minlength=num_state_sets).astype(np.uint32)
    return TierAImage(img, base, level, int(root), np.ascontiguousarray(d), counts, H)


def slot_layout(counts, seed: int):
    """A slot layout (the input of the device-resident StateSet packing)
    whose packing is a given grouping: region j of the packed array
    (counts[j] records) belongs to StateSet dfs[j], and slot k holds the
    record of packed position perm[k], a seeded random permutation.
    Returns (dfs, state_set_of_slot, list_index_of_slot, perm, region
    starts)."""
    counts = np.asarray(counts, np.int64)
    S, n = len(counts), int(counts.sum())
    rs = np.random.default_rng(seed)
    dfs = rs.permutation(S).astype(np.uint32)
    starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    region_of_pos = np.repeat(np.arange(S), counts)
    perm = rs.permutation(n)
    set_of_slot = dfs[region_of_pos[perm]].astype(np.uint32)
    list_index = (perm - starts[region_of_pos[perm]]).astype(np.uint32)
    return dfs, set_of_slot, list_index, perm, starts.astype(np.uint32)
