// scene.cu - Tier B scenes: device-resident structure-of-arrays storage,
// host uploads through the context's side stream, and the plain pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "capi_internal.h"

using namespace cadr;

namespace cadr {

ViewConst to_view_const(const cadr_view& v)
{
    ViewConst c;
    std::memcpy(&c, &v, sizeof(c));
    return c;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static cadr_status before_upload(cadr_scene* sc);
static cadr_status after_upload(cadr_scene* sc);

// The plain pass's per-tile tables: for each leaf tile of kLeafTile
// drawables, the start of the StateSet region holding its last drawable
// (for the stream kernel) and the regions of its first and last drawable,
// clamped to S-1 (for the write kernels): the region searches a CTA would
// otherwise make.  Built on the host from the validated offsets at every
// commit, uploaded on the upload stream.
static cadr_status upload_tile_starts(cadr_scene* sc)
{
    const uint64_t N = sc->desc.num_drawables;
    const uint32_t S = sc->desc.num_state_sets;
    const std::vector<uint32_t>& off = sc->h_offsets;
    const uint64_t tiles = (N + kLeafTile - 1) / kLeafTile;
    sc->h_tile_start.resize(tiles);
    sc->h_tile_region.resize(tiles * 2);
    auto region = [&](uint32_t key) {
        size_t r = (size_t)(std::upper_bound(off.begin(), off.end(), key) - off.begin()) - 1;
        return (uint32_t)std::min<size_t>(r, S - 1);
    };
    for (uint64_t t = 0; t < tiles; t++) {
        const uint32_t first = (uint32_t)(t * kLeafTile);
        const uint32_t last = (uint32_t)(std::min<uint64_t>((t + 1) * kLeafTile, N) - 1);
        const uint32_t rl = region(last);
        sc->h_tile_start[t] = off[rl];
        sc->h_tile_region[2 * t] = region(first);
        sc->h_tile_region[2 * t + 1] = rl;
    }
    if (tiles == 0) return CADR_OK;
    cadr_status st = before_upload(sc);
    if (st == CADR_OK)
        st = upload_bytes(sc->ctx, sc->tile_start, sc->h_tile_start.data(), tiles * 4, sc->ctx->upload_stream);
    if (st == CADR_OK)
        st = upload_bytes(sc->ctx, sc->tile_region, sc->h_tile_region.data(), tiles * 8, sc->ctx->upload_stream);
    if (st != CADR_OK) return st;
    return after_upload(sc);
}

static cadr_status commit(cadr_scene* sc)
{
    const uint32_t S = sc->desc.num_state_sets;
    std::vector<uint32_t> off(S + 1);
    cudaError_t e = cudaStreamSynchronize(sc->ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(off.data(), sc->buf.state_set_offsets, (S + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "scene_commit: read offsets");
    if (off[0] != 0 || off[S] != sc->desc.num_drawables)
        return fail(CADR_ERR_INVALID_ARG, "scene_commit: StateSet offsets must start at 0 and end at %llu",
                    (unsigned long long)sc->desc.num_drawables);
    for (uint32_t s = 0; s < S; s++)
        if (off[s + 1] < off[s]) return fail(CADR_ERR_INVALID_ARG, "scene_commit: StateSet offsets not sorted at %u", s);
    sc->h_offsets = std::move(off);
    cadr_status st = upload_tile_starts(sc);
    if (st != CADR_OK) return st;
    sc->committed = true;
    return CADR_OK;
}

cadr_status scene_prepare(cadr_scene* sc, cudaStream_t stream)
{
    if (!sc->committed) {
        cadr_status st = commit(sc);
        if (st != CADR_OK) return st;
    }
    if (sc->upload_pending) {
        cudaError_t e = cudaStreamWaitEvent(stream, sc->uploaded, 0);
        if (e != cudaSuccess) return cuda_fail(e, "scene: wait for uploads");
    }
    return CADR_OK;
}

cadr_status scene_mark_read(cadr_scene* sc, cudaStream_t stream)
{
    cudaError_t e = cudaEventRecord(sc->read_done, stream);
    if (e != cudaSuccess) return cuda_fail(e, "scene: record read");
    sc->read_pending = true;
    return CADR_OK;
}

// Uploads go to the context's upload stream; an upload into a scene waits
// there for the passes issued before it that read the scene.
static cadr_status before_upload(cadr_scene* sc)
{
    if (!sc->read_pending) return CADR_OK;
    cudaError_t e = cudaStreamWaitEvent(sc->ctx->upload_stream, sc->read_done, 0);
    if (e != cudaSuccess) return cuda_fail(e, "scene upload: wait for readers");
    return CADR_OK;
}

static cadr_status after_upload(cadr_scene* sc)
{
    cudaError_t e = cudaEventRecord(sc->uploaded, sc->ctx->upload_stream);
    if (e != cudaSuccess) return cuda_fail(e, "scene upload: record");
    sc->upload_pending = true;
    return CADR_OK;
}

// Propagation of the internal levels 1..L-1 (level 0's world is its local).
cadr_status propagate_levels(cadr_scene* sc, cudaStream_t stream, cudaEvent_t* level_events)
{
    cadr_context* ctx = sc->ctx;
    const cadr_scene_desc& d = sc->desc;
    // Leading levels small enough to hold in one CTA's shared memory (two
    // at least) are folded into one launch.
    uint32_t fold = 0;
    if (d.num_levels >= 3) {
        uint64_t nodes = d.level_size[0];
        while (1 + fold < d.num_levels && nodes + d.level_size[1 + fold] <= kFoldMaxNodes)
            nodes += d.level_size[1 + fold++];
        if (fold < 2) fold = 0;
    }
    if (fold) {
        FoldArgs f{};
        f.world0 = reinterpret_cast<const float4*>(sc->buf.level_world[0]);
        f.n0 = (uint32_t)d.level_size[0];
        f.count = fold;
        for (uint32_t k = 0; k < fold; k++) {
            f.lvl[k].local = reinterpret_cast<const float4*>(sc->buf.level_local[1 + k]);
            f.lvl[k].parent = sc->buf.level_parent[1 + k];
            f.lvl[k].world = reinterpret_cast<float4*>(sc->buf.level_world[1 + k]);
            f.lvl[k].n = (uint32_t)d.level_size[1 + k];
        }
        f.error = ctx->d_error;
        f.limit_ns = ctx->spin_limit_ns;
        cudaError_t e = launch_small_levels(f, stream);
        if (e != cudaSuccess) return cuda_fail(e, "propagate: launch folded levels");
        ctx->launches++;
        // Frame timing gives the folded launch to its first level.
        for (uint32_t k = 0; level_events && k < fold; k++) {
            e = cudaEventRecord(level_events[1 + k], stream);
            if (e != cudaSuccess) return cuda_fail(e, "propagate: level event");
        }
    }
    for (uint32_t l = 1 + fold; l < d.num_levels; l++) {
        cudaError_t e = launch_propagate(
            reinterpret_cast<const float4*>(sc->buf.level_world[l - 1]), (uint32_t)sc->desc.level_size[l - 1],
            reinterpret_cast<const float4*>(sc->buf.level_local[l]), sc->buf.level_parent[l],
            (uint32_t)sc->desc.level_size[l], reinterpret_cast<float4*>(sc->buf.level_world[l]), 1,
            ctx->d_error, ctx->spin_limit_ns, stream, l >= 2 && !level_events);
        if (e != cudaSuccess) return cuda_fail(e, "propagate: launch");
        if (sc->desc.level_size[l]) ctx->launches++;
        if (level_events) {
            e = cudaEventRecord(level_events[l], stream);
            if (e != cudaSuccess) return cuda_fail(e, "propagate: level event");
        }
    }
    return CADR_OK;
}

LeafArgs leaf_args(cadr_scene* sc)
{
    const cadr_scene_desc& d = sc->desc;
    LeafArgs a{};
    a.local = reinterpret_cast<const float4*>(sc->buf.local);
    a.parent = d.num_levels ? sc->buf.parent : nullptr;
    a.parent_world = d.num_levels ? reinterpret_cast<const float4*>(sc->buf.level_world[d.num_levels - 1]) : nullptr;
    a.num_parents = d.num_levels ? (uint32_t)d.level_size[d.num_levels - 1] : 0;
    a.sphere = reinterpret_cast<const float4*>(sc->buf.sphere);
    a.geometry = sc->buf.geometry;
    a.offsets = sc->buf.state_set_offsets;
    a.tile_start = sc->tile_start;
    a.tile_region = reinterpret_cast<const uint2*>(sc->tile_region);
    a.num_state_sets = d.num_state_sets;
    a.lods = reinterpret_cast<const uint4*>(sc->buf.lods);
    a.num_geometries = d.num_geometries;
    a.num_lods = d.num_lods;
    a.n = (uint32_t)d.num_drawables;
    a.world = reinterpret_cast<float4*>(sc->buf.world);
    a.world_sphere = nullptr;
    a.error = sc->ctx->d_error;
    return a;
}

}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_scene_create(cadr_context* ctx, const cadr_scene_desc* desc, cadr_scene** out)
{
    if (!ctx || !desc || !out) return fail(CADR_ERR_INVALID_ARG, "scene_create: null argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    const cadr_scene_desc& d = *desc;
    if (d.num_levels > CADR_MAX_LEVELS) return fail(CADR_ERR_INVALID_ARG, "scene_create: too many levels");
    if (d.num_state_sets == 0 || d.num_geometries == 0 || d.num_lods < 1 || d.num_lods > 4)
        return fail(CADR_ERR_INVALID_ARG, "scene_create: need >= 1 StateSet and geometry, 1..4 LODs");
    if (d.num_drawables > 0xFFFF0000ull) return fail(CADR_ERR_INVALID_ARG, "scene_create: too many drawables");
    for (uint32_t l = 0; l < d.num_levels; l++)
        if (d.level_size[l] == 0 || d.level_size[l] > 0xFFFF0000ull)
            return fail(CADR_ERR_INVALID_ARG, "scene_create: level %u size out of range", l);
    const uint64_t N = d.num_drawables;
    // Arena layout.
    size_t off = 0;
    size_t lvl_local[CADR_MAX_LEVELS], lvl_parent[CADR_MAX_LEVELS], lvl_world[CADR_MAX_LEVELS];
    for (uint32_t l = 0; l < d.num_levels; l++) {
        const uint64_t n = d.level_size[l];
        lvl_local[l] = off; off = align256(off + n * 64);
        lvl_parent[l] = off; if (l) off = align256(off + n * 4);
        lvl_world[l] = off; if (l) off = align256(off + n * 64);
    }
    const size_t o_local = off; off = align256(off + N * 64);
    const size_t o_parent = off; off = align256(off + (d.num_levels ? N * 4 : 0));
    const size_t o_sphere = off; off = align256(off + N * 16);
    const size_t o_geom = off; off = align256(off + N * 4);
    const size_t o_offsets = off; off = align256(off + (size_t)(d.num_state_sets + 1) * 4);
    const size_t o_lods = off; off = align256(off + (size_t)d.num_geometries * d.num_lods * 16);
    const size_t o_world = off; off = align256(off + N * 64);
    const size_t o_wsph = off; off = align256(off + N * 16);
    const size_t o_tiles = off; off = align256(off + (N + kLeafTile - 1) / kLeafTile * 4);
    const size_t o_treg = off; off = align256(off + (N + kLeafTile - 1) / kLeafTile * 8);

    auto* sc = new cadr_scene();
    sc->ctx = ctx;
    sc->desc = d;
    cudaError_t e = cudaMalloc(&sc->arena, off ? off : 256);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sc->uploaded, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sc->read_done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cadr_scene_destroy(sc);
        return cuda_fail(e, "scene_create: device memory");
    }
    sc->arena_bytes = off;
    uint8_t* base = static_cast<uint8_t*>(sc->arena);
    for (uint32_t l = 0; l < d.num_levels; l++) {
        sc->buf.level_local[l] = reinterpret_cast<float*>(base + lvl_local[l]);
        sc->buf.level_parent[l] = l ? reinterpret_cast<uint32_t*>(base + lvl_parent[l]) : nullptr;
        sc->buf.level_world[l] = l ? reinterpret_cast<float*>(base + lvl_world[l]) : sc->buf.level_local[0];
    }
    sc->buf.local = reinterpret_cast<float*>(base + o_local);
    sc->buf.parent = d.num_levels ? reinterpret_cast<uint32_t*>(base + o_parent) : nullptr;
    sc->buf.sphere = reinterpret_cast<float*>(base + o_sphere);
    sc->buf.geometry = reinterpret_cast<uint32_t*>(base + o_geom);
    sc->buf.state_set_offsets = reinterpret_cast<uint32_t*>(base + o_offsets);
    sc->buf.lods = reinterpret_cast<cadr_lod*>(base + o_lods);
    sc->buf.world = reinterpret_cast<float*>(base + o_world);
    sc->buf.world_sphere = reinterpret_cast<float*>(base + o_wsph);
    sc->tile_start = reinterpret_cast<uint32_t*>(base + o_tiles);
    sc->tile_region = reinterpret_cast<uint32_t*>(base + o_treg);
    // Defaults: all drawables in StateSet 0 until offsets are uploaded.
    std::vector<uint32_t> off0(d.num_state_sets + 1, (uint32_t)N);
    off0[0] = 0;
    e = cudaMemcpy(sc->buf.state_set_offsets, off0.data(), off0.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cadr_scene_destroy(sc);
        return cuda_fail(e, "scene_create: init offsets");
    }
    *out = sc;
    return CADR_OK;
}

CADR_API cadr_status cadr_scene_destroy(cadr_scene* sc)
{
    if (!sc) return CADR_OK;
    DeviceGuard dg(sc->ctx->device);
    if (sc->ctx->shard_scene == sc) sc->ctx->shard_scene = nullptr;
    cudaDeviceSynchronize();
    if (sc->arena) cudaFree(sc->arena);
    if (sc->uploaded) cudaEventDestroy(sc->uploaded);
    if (sc->read_done) cudaEventDestroy(sc->read_done);
    delete sc;
    return CADR_OK;
}

CADR_API cadr_status cadr_scene_get_buffers(cadr_scene* sc, cadr_scene_buffers* out)
{
    if (!sc || !out) return fail(CADR_ERR_INVALID_ARG, "scene_get_buffers: null argument");
    *out = sc->buf;
    sc->committed = false;  // the caller may write in place; re-validate before the next pass
    return CADR_OK;
}

CADR_API cadr_status cadr_scene_upload_level(cadr_scene* sc, uint32_t level, const float* local,
                                             const uint32_t* parent, uint64_t first, uint64_t count)
{
    if (!sc || level >= sc->desc.num_levels) return fail(CADR_ERR_INVALID_ARG, "scene_upload_level: bad level");
    DeviceGuard dg(sc->ctx->device);
    const uint64_t n = sc->desc.level_size[level];
    if (first > n || count > n - first) return fail(CADR_ERR_INVALID_ARG, "scene_upload_level: rows out of range");
    if (level == 0 && parent) return fail(CADR_ERR_INVALID_ARG, "scene_upload_level: level 0 has no parents");
    cadr_context* ctx = sc->ctx;
    cadr_status st = before_upload(sc);
    if (st != CADR_OK) return st;
    if (local) st = upload_bytes(ctx, sc->buf.level_local[level] + first * 16, local, count * 64, ctx->upload_stream);
    if (st == CADR_OK && parent)
        st = upload_bytes(ctx, sc->buf.level_parent[level] + first, parent, count * 4, ctx->upload_stream);
    if (st != CADR_OK) return st;
    return after_upload(sc);
}

CADR_API cadr_status cadr_scene_upload_drawables(cadr_scene* sc, const float* local, const uint32_t* parent,
                                                 const float* sphere, const uint32_t* geometry, uint64_t first,
                                                 uint64_t count)
{
    if (!sc) return fail(CADR_ERR_INVALID_ARG, "scene_upload_drawables: null scene");
    DeviceGuard dg(sc->ctx->device);
    const uint64_t n = sc->desc.num_drawables;
    if (first > n || count > n - first) return fail(CADR_ERR_INVALID_ARG, "scene_upload_drawables: rows out of range");
    if (parent && !sc->desc.num_levels) return fail(CADR_ERR_INVALID_ARG, "scene_upload_drawables: scene has no hierarchy");
    cadr_context* ctx = sc->ctx;
    cadr_status st = before_upload(sc);
    if (st != CADR_OK) return st;
    if (local) st = upload_bytes(ctx, sc->buf.local + first * 16, local, count * 64, ctx->upload_stream);
    if (st == CADR_OK && parent) st = upload_bytes(ctx, sc->buf.parent + first, parent, count * 4, ctx->upload_stream);
    if (st == CADR_OK && sphere) st = upload_bytes(ctx, sc->buf.sphere + first * 4, sphere, count * 16, ctx->upload_stream);
    if (st == CADR_OK && geometry)
        st = upload_bytes(ctx, sc->buf.geometry + first, geometry, count * 4, ctx->upload_stream);
    if (st != CADR_OK) return st;
    return after_upload(sc);
}

CADR_API cadr_status cadr_scene_upload_state_sets(cadr_scene* sc, const uint32_t* offsets)
{
    if (!sc || !offsets) return fail(CADR_ERR_INVALID_ARG, "scene_upload_state_sets: null argument");
    DeviceGuard dg(sc->ctx->device);
    const uint32_t S = sc->desc.num_state_sets;
    if (offsets[0] != 0 || offsets[S] != sc->desc.num_drawables)
        return fail(CADR_ERR_INVALID_ARG, "scene_upload_state_sets: offsets must start at 0 and end at N");
    for (uint32_t s = 0; s < S; s++)
        if (offsets[s + 1] < offsets[s]) return fail(CADR_ERR_INVALID_ARG, "scene_upload_state_sets: offsets not sorted");
    cadr_status st = before_upload(sc);
    if (st == CADR_OK) st = upload_bytes(sc->ctx, sc->buf.state_set_offsets, offsets, (size_t)(S + 1) * 4, sc->ctx->upload_stream);
    if (st != CADR_OK) return st;
    sc->committed = false;
    return after_upload(sc);
}

CADR_API cadr_status cadr_scene_upload_lods(cadr_scene* sc, const cadr_lod* lods)
{
    if (!sc || !lods) return fail(CADR_ERR_INVALID_ARG, "scene_upload_lods: null argument");
    DeviceGuard dg(sc->ctx->device);
    cadr_status st = before_upload(sc);
    if (st != CADR_OK) return st;
    st = upload_bytes(sc->ctx, sc->buf.lods, lods,
                                  (size_t)sc->desc.num_geometries * sc->desc.num_lods * 16, sc->ctx->upload_stream);
    if (st != CADR_OK) return st;
    return after_upload(sc);
}

CADR_API cadr_status cadr_scene_commit(cadr_scene* sc)
{
    if (!sc) return fail(CADR_ERR_INVALID_ARG, "scene_commit: null scene");
    DeviceGuard dg(sc->ctx->device);
    return commit(sc);
}

CADR_API cadr_status cadr_scene_propagate(cadr_scene* sc, int write_world_spheres, cadr_stream stream)
{
    if (!sc) return fail(CADR_ERR_INVALID_ARG, "scene_propagate: null scene");
    DeviceGuard dg(sc->ctx->device);
    cudaStream_t s = pick_stream(sc->ctx, stream);
    cadr_status st = scene_prepare(sc, s);
    if (st != CADR_OK) return st;
    st = propagate_levels(sc, s);
    if (st != CADR_OK) return st;
    LeafArgs a = leaf_args(sc);
    if (write_world_spheres) a.world_sphere = reinterpret_cast<float4*>(sc->buf.world_sphere);
    cudaError_t e = launch_leaf_propagate(a, s);
    if (e != cudaSuccess) return cuda_fail(e, "scene_propagate: launch");
    if (a.n) sc->ctx->launches++;
    return scene_mark_read(sc, s);
}

CADR_API cadr_status cadr_cull(cadr_scene* sc, const cadr_view* view, cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                               uint32_t* marginal, cadr_stream stream)
{
    if (!sc || !view || !counts || (!cmds && sc->desc.num_drawables))
        return fail(CADR_ERR_INVALID_ARG, "cull: null argument");
    DeviceGuard dg(sc->ctx->device);
    cadr_context* ctx = sc->ctx;
    cudaStream_t s = pick_stream(ctx, stream);
    cadr_status st = scene_prepare(sc, s);
    if (st != CADR_OK) return st;
    cudaError_t e;
    if (sc->desc.num_drawables == 0) {
        e = cudaMemsetAsync(counts, 0, (size_t)sc->desc.num_state_sets * 4, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull: clear counts");
        return CADR_OK;
    }
    const uint64_t tiles = (sc->desc.num_drawables + kLeafTile - 1) / kLeafTile;
    st = scratch_reserve(ctx, ctx->scratch, tiles);
    if (st == CADR_OK) st = scratch_reserve_planes(ctx, ctx->scratch, leaf_plane_words(sc->desc.num_drawables));
    if (st != CADR_OK) return st;
    if (ctx->pass_recorded) {
        e = cudaStreamWaitEvent(s, ctx->pass_done, 0);
        if (e != cudaSuccess) return cuda_fail(e, "cull: order after previous pass");
    }
    cudaEvent_t* fev = nullptr;
    cudaEvent_t* lev = nullptr;
    if (ctx->collect_frames) {
        if (ctx->frame_head - ctx->frame_tail == (uint64_t)cadr_context::kFrames) ctx->frame_tail++;
        const uint64_t f = ctx->frame_head % cadr_context::kFrames;
        fev = ctx->frame_ev[f];
        lev = ctx->level_ev[f];
        ctx->frame_levels[f] = sc->desc.num_levels;
        cudaEventRecord(fev[0], s);
    }
    st = propagate_levels(sc, s, lev);
    if (st != CADR_OK) return st;
    if (fev) cudaEventRecord(fev[1], s);
    LeafArgs a = leaf_args(sc);
    a.cmds = reinterpret_cast<uint32_t*>(cmds);
    a.counts = counts;
    a.marginal = marginal;
    a.view = to_view_const(*view);
    // The stream kernel overlaps the last level kernel's tail when that
    // kernel is the launch just before it (no frame-timing event between).
    e = launch_leaf_cull(a, ctx->scratch, s, fev ? fev[2] : nullptr, !fev && sc->desc.num_levels >= 2);
    if (e != cudaSuccess) return cuda_fail(e, "cull: launch");
    ctx->launches += kLeafCullLaunches;
    if (fev) {
        cudaEventRecord(fev[3], s);
        ctx->frame_head++;
    }
    ctx->scratch.launches++;
    e = cudaEventRecord(ctx->pass_done, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull: record");
    ctx->pass_recorded = true;
    return scene_mark_read(sc, s);
}

}  // extern "C"
