// shard.cu - the plain pass over one shard of a scene whose drawables are
// split over several devices, in two phases around the one exchange step.
//
// A shard is a contiguous range [lo, hi) of the StateSet-grouped drawables,
// held as its own scene (its drawables, the replicated internal levels, its
// StateSet offsets clipped to the range).  Phase 1 (cadr_cull_shard_count)
// runs propagation, the stream kernel and the tile scan, and counts the
// visible drawables of every StateSet region.  The ranks exchange these
// counts (an all-gather of S words); rank r's commands of region s then
// start at offsets[s] + sum_{q<r} count[q][s] of the merged buffer.  Phase 2
// (cadr_cull_shard_write) runs the write kernel with those destination
// bases and firstInstance offset by lo, so the merged buffer equals the
// single-device pass word for word.  The planes and tile carries live in
// the context's shard scratch between the phases.
#include <cuda_runtime.h>

#include "capi_internal.h"

using namespace cadr;

extern "C" {

CADR_API cadr_status cadr_cull_shard_count(cadr_scene* sc, const cadr_view* view, uint32_t* counts,
                                           uint32_t* marginal, cadr_stream stream)
{
    if (!sc || !view || !counts) return fail(CADR_ERR_INVALID_ARG, "cull_shard_count: null argument");
    DeviceGuard dg(sc->ctx->device);
    cadr_context* ctx = sc->ctx;
    cudaStream_t s = pick_stream(ctx, stream);
    cadr_status st = scene_prepare(sc, s);
    if (st != CADR_OK) return st;
    cudaError_t e;
    if (sc->desc.num_drawables == 0) {
        e = cudaMemsetAsync(counts, 0, (size_t)sc->desc.num_state_sets * 4, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_shard_count: clear counts");
        ctx->shard_scene = sc;
        e = cudaEventRecord(ctx->shard_counted, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_shard_count: record");
        return CADR_OK;
    }
    const uint64_t tiles = (sc->desc.num_drawables + kLeafTile - 1) / kLeafTile;
    // A new count phase replaces a pending one: the write of that one must
    // not read this one's scratch.
    ctx->shard_scene = nullptr;
    st = scratch_reserve(ctx, ctx->shard_scratch, tiles);
    if (st == CADR_OK) st = scratch_reserve_planes(ctx, ctx->shard_scratch, leaf_plane_words(sc->desc.num_drawables));
    if (st != CADR_OK) return st;
    // Ordered after the context's previous plain pass (passes over a scene
    // rewrite its world matrices) and after the previous shard write, which
    // reads the shard scratch this phase rewrites.
    if (ctx->pass_recorded) {
        e = cudaStreamWaitEvent(s, ctx->pass_done, 0);
        if (e != cudaSuccess) return cuda_fail(e, "cull_shard_count: order after previous pass");
    }
    st = propagate_levels(sc, s);
    if (st != CADR_OK) return st;
    LeafArgs a = leaf_args(sc);
    a.counts = counts;
    a.marginal = marginal;
    a.view = to_view_const(*view);
    e = launch_leaf_stream_scan(a, ctx->shard_scratch, s, nullptr, sc->desc.num_levels >= 2);
    if (e == cudaSuccess) e = launch_leaf_region_counts(a, ctx->shard_scratch, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull_shard_count: launch");
    ctx->launches += 3;
    e = cudaEventRecord(ctx->shard_counted, s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->pass_done, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull_shard_count: record");
    ctx->pass_recorded = true;
    ctx->shard_scene = sc;
    return scene_mark_read(sc, s);
}

CADR_API cadr_status cadr_cull_shard_write(cadr_scene* sc, const uint32_t* dst_base, uint32_t first_instance,
                                           cadr_draw_indexed_cmd* cmds, uint64_t cmd_capacity, cadr_stream stream)
{
    if (!sc || (sc->desc.num_drawables && (!dst_base || !cmds)))
        return fail(CADR_ERR_INVALID_ARG, "cull_shard_write: null argument");
    DeviceGuard dg(sc->ctx->device);
    cadr_context* ctx = sc->ctx;
    if (ctx->shard_scene != sc)
        return fail(CADR_ERR_INVALID_ARG, "cull_shard_write: no count phase of this scene is pending "
                                          "(call cadr_cull_shard_count first)");
    if (cmd_capacity > 0xffffffffull || (uint64_t)first_instance + sc->desc.num_drawables > 0x100000000ull)
        return fail(CADR_ERR_INVALID_ARG, "cull_shard_write: command indices beyond 32 bits");
    cudaStream_t s = pick_stream(ctx, stream);
    ctx->shard_scene = nullptr;
    if (sc->desc.num_drawables == 0) return CADR_OK;
    cudaError_t e = cudaStreamWaitEvent(s, ctx->shard_counted, 0);
    if (e != cudaSuccess) return cuda_fail(e, "cull_shard_write: order after the count phase");
    LeafArgs a = leaf_args(sc);
    a.cmds = reinterpret_cast<uint32_t*>(cmds);
    a.shard.dst_base = dst_base;
    a.shard.first_instance = first_instance;
    a.shard.capacity = (uint32_t)cmd_capacity;
    e = launch_leaf_write(a, ctx->shard_scratch, s, false);
    if (e != cudaSuccess) return cuda_fail(e, "cull_shard_write: launch");
    ctx->launches += 1;
    e = cudaEventRecord(ctx->pass_done, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull_shard_write: record");
    ctx->pass_recorded = true;
    return scene_mark_read(sc, s);
}

}  // extern "C"
