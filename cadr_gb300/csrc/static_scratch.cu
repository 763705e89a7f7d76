// static_scratch.cu - the plain pass with its scratch memory in a statically
// allocated device array, for callers that cannot allocate device memory.
//
// cadr_cull keeps its scratch (one word per tile of 2,048 drawables and
// three bit-planes of one word per 32 drawables) in memory it allocates
// with cudaMalloc, and grows it, after a device-wide synchronisation, when
// a scene needs more than it holds.  Some
// callers cannot let that happen: a renderer whose device memory is owned
// and budgeted by the host application (every buffer imported or carved
// out at start-up), or a frame loop that must not stall, since cudaMalloc
// and cudaFree synchronise the device.  cadr_cull_static_scratch runs the
// same kernels, with the same results, but takes its scratch from the
// file-scope array below, which exists on every device that loads this
// library until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "capi_internal.h"

using namespace cadr;

namespace cadr {
namespace {

// Largest scene the entry point accepts, and the tiles it needs.
constexpr uint64_t kStaticMaxDrawables = 33554432;
constexpr uint64_t kStaticMaxTiles = (kStaticMaxDrawables + kLeafTile - 1) / kLeafTile;
constexpr size_t kTileBytes = kStaticMaxTiles * sizeof(uint64_t);                       // 128 KiB
constexpr size_t kPlaneBytes = leaf_plane_words(kStaticMaxDrawables) * sizeof(uint32_t);  // 12 MiB
constexpr size_t kStaticScratchBytes = kTileBytes + kPlaneBytes;

// The scratch.  Host code must not take this symbol's address directly: on
// the host it names a stand-in, not device memory.  The device address comes
// from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_address[kMaxDevices] = {};

// Set-up on the first call per device.  The caller (the entry point, under
// its DeviceGuard) has made `device` current, so the symbol's address is
// that device's copy of the array; the guard gives the calling thread its
// own device back afterwards, on the error paths too.
cadr_status static_scratch_address(int device, void** out)
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (device < 0 || device >= kMaxDevices)
        return fail(CADR_ERR_INVALID_ARG, "cull_static_scratch: device %d out of range", device);
    if (!g_scratch_address[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cull_static_scratch: scratch address");
        g_scratch_address[device] = p;
    }
    *out = g_scratch_address[device];
    return CADR_OK;
}

}  // namespace
}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_cull_static_scratch(cadr_scene* sc, const cadr_view* view, cadr_draw_indexed_cmd* cmds,
                                              uint32_t* counts, uint32_t* marginal, cadr_stream stream)
{
    if (!sc || !view || !counts || (!cmds && sc->desc.num_drawables))
        return fail(CADR_ERR_INVALID_ARG, "cull_static_scratch: null argument");
    DeviceGuard dg(sc->ctx->device);
    if (!sc->committed)
        return fail(CADR_ERR_INVALID_ARG, "cull_static_scratch: commit the scene (cadr_scene_commit) first");
    if (sc->desc.num_drawables > kStaticMaxDrawables)
        return fail(CADR_ERR_INVALID_ARG, "cull_static_scratch: %llu drawables exceed the maximum of %llu",
                    (unsigned long long)sc->desc.num_drawables, (unsigned long long)kStaticMaxDrawables);
    cadr_context* ctx = sc->ctx;
    void* base = nullptr;
    cadr_status st = static_scratch_address(ctx->device, &base);
    if (st != CADR_OK) return st;
    cudaStream_t s = pick_stream(ctx, stream);
    st = scene_prepare(sc, s);
    if (st != CADR_OK) return st;
    cudaError_t e;
    if (sc->desc.num_drawables == 0) {
        e = cudaMemsetAsync(counts, 0, (size_t)sc->desc.num_state_sets * 4, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_static_scratch: clear counts");
        return CADR_OK;
    }
    // Every word of the tile states and planes that a pass reads, the pass
    // writes first: the array needs no clearing between calls.
    Scratch scratch;
    scratch.tile_state = static_cast<uint64_t*>(base);
    scratch.capacity = kStaticMaxTiles;
    scratch.planes = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + kTileBytes);
    scratch.plane_words = leaf_plane_words(kStaticMaxDrawables);
    // Ordered after the context's previous plain pass (cadr_cull or this
    // entry point, on any stream), as cadr_cull is: passes over one scene
    // rewrite its world matrices.  Waiting on and recording an event
    // allocates nothing.
    if (ctx->pass_recorded) {
        e = cudaStreamWaitEvent(s, ctx->pass_done, 0);
        if (e != cudaSuccess) return cuda_fail(e, "cull_static_scratch: order after previous pass");
    }
    st = propagate_levels(sc, s);
    if (st != CADR_OK) return st;
    LeafArgs a = leaf_args(sc);
    a.cmds = reinterpret_cast<uint32_t*>(cmds);
    a.counts = counts;
    a.marginal = marginal;
    a.view = to_view_const(*view);
    // The same launch sequence as cadr_cull: the stream kernel is a
    // programmatic dependent of the last level kernel when there is one.
    e = launch_leaf_cull(a, scratch, s, nullptr, sc->desc.num_levels >= 2);
    if (e != cudaSuccess) return cuda_fail(e, "cull_static_scratch: launch");
    ctx->launches += kLeafCullLaunches;
    e = cudaEventRecord(ctx->pass_done, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull_static_scratch: record");
    ctx->pass_recorded = true;
    return scene_mark_read(sc, s);
}

}  // extern "C"
