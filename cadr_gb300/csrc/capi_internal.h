// capi_internal.h - internal state behind the opaque C ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "device_guard.h"
#include "kernels.cuh"

namespace cadr {
constexpr int kRingSlots = 2;
// L2 fetch granularity the context sets for the process (bytes).
constexpr size_t kL2FetchBytes = 32;
struct BatchedState;
}

struct cadr_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;         // default compute stream
    cudaStream_t upload_stream = nullptr;  // side stream of staged uploads
    cudaEvent_t upload_done = nullptr;
    cudaEvent_t pass_done = nullptr;       // orders passes sharing `scratch`
    bool pass_recorded = false;
    cudaEvent_t ring_event[cadr::kRingSlots] = {};
    uint8_t* ring = nullptr;               // pinned staging ring
    size_t ring_bytes = size_t(64) << 20;
    int ring_next = 0;
    std::mutex ring_mu;
    size_t prev_l2_fetch = 0;              // the device's L2 fetch granularity before this context
    bool l2_fetch_set = false;
    uint32_t* h_error = nullptr;           // mapped pinned error word
    uint32_t* d_error = nullptr;
    uint64_t spin_limit_ns = 1000000000ull;
    uint32_t fault = 0;
    std::atomic<uint64_t> launches{0};
    cadr::Scratch scratch;                 // lookback scratch of plain passes
    cadr::Scratch shard_scratch;           // planes and tile carries kept from a shard's count to its write
    cudaEvent_t shard_counted = nullptr;   // recorded after a shard's count phase
    cadr_scene* shard_scene = nullptr;     // the scene whose shard pass awaits its write phase
    cadr_tuning tuning = {256, 4, 4, 0};
    std::string tuning_cache;              // autotuner cache file ("" = none)
    cadr::BatchedState* batched = nullptr;
    // frame timing ring (cadr_frame_info)
    static constexpr int kFrames = 256;
    bool collect_frames = false;
    cudaEvent_t frame_ev[kFrames][4] = {};  // before levels, after levels, after stream kernel, after leaf stage
    cudaEvent_t level_ev[kFrames][CADR_MAX_LEVELS] = {};  // after level l's propagation (l >= 1)
    uint32_t frame_levels[kFrames] = {};
    // Timestamps of the facade's frames (cadr_context_record_timestamp):
    // four per frame, for the last kTsFrames frames.
    static constexpr int kTsFrames = 4;
    cudaEvent_t ts_ev[kTsFrames][4] = {};
    uint64_t ts_frame[kTsFrames] = {~0ull, ~0ull, ~0ull, ~0ull};
    uint32_t ts_mask[kTsFrames] = {};
    uint64_t frame_head = 0, frame_tail = 0;
};

struct cadr_scene {
    cadr_context* ctx = nullptr;
    cadr_scene_desc desc = {};
    void* arena = nullptr;
    size_t arena_bytes = 0;
    cadr_scene_buffers buf = {};
    std::vector<uint32_t> h_offsets;       // host copy of the StateSet offsets
    std::vector<uint32_t> h_tile_start;    // per leaf tile: start of the region of its last drawable
    uint32_t* tile_start = nullptr;        // device copy of h_tile_start (in the arena)
    std::vector<uint32_t> h_tile_region;   // per leaf tile: regions of its first and last drawable
    uint32_t* tile_region = nullptr;       // device copy of h_tile_region (in the arena)
    bool committed = false;
    bool upload_pending = false;
    cudaEvent_t uploaded = nullptr;
    bool read_pending = false;
    cudaEvent_t read_done = nullptr;       // recorded after the last pass that reads the scene
};

namespace cadr {
extern thread_local std::string g_last_error;
cadr_status fail(cadr_status s, const char* fmt, ...);
cadr_status cuda_fail(cudaError_t e, const char* what);
cadr_status scratch_reserve(cadr_context* ctx, Scratch& s, uint64_t tiles);
// Grows s.planes to at least `words` (after a device-wide synchronisation).
cadr_status scratch_reserve_planes(cadr_context* ctx, Scratch& s, uint64_t words);
void scratch_release(Scratch& s);
cadr_status upload_bytes(cadr_context* ctx, void* dst, const void* src, size_t bytes, cudaStream_t stream);
cudaStream_t pick_stream(cadr_context* ctx, cadr_stream s);
void destroy_batched_state(cadr_context* ctx);
cadr_status scene_prepare(cadr_scene* sc, cudaStream_t stream);
// After a pass on `stream` that reads the scene: later uploads into the
// scene wait for it.
cadr_status scene_mark_read(cadr_scene* sc, cudaStream_t stream);
ViewConst to_view_const(const cadr_view& v);
cadr_status build_jobs(const cadr_batch_view* views, uint32_t n, uint32_t tile, ViewJob* jobs, uint64_t* total);
// Propagation of the internal levels 1..L-1 on `stream`, each level a
// programmatic dependent of the one before.  With `level_events`, the
// event of level l is recorded after its launch and the levels run one
// after the other (frame timing).
cadr_status propagate_levels(cadr_scene* sc, cudaStream_t stream, cudaEvent_t* level_events = nullptr);
LeafArgs leaf_args(cadr_scene* sc);
}  // namespace cadr
