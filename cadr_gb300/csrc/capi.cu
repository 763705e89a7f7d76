// capi.cu - the C ABI of libcadr_cuda.so: contexts, device/pinned memory,
// stream-ordered uploads through a pinned staging ring on a side stream,
// Tier A dispatch and Tier B scenes and plain passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace cadr;

namespace cadr {

thread_local std::string g_last_error;

cadr_status fail(cadr_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

cadr_status cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(CADR_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(CADR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

cadr_status scratch_reserve_planes(cadr_context* ctx, Scratch& s, uint64_t words)
{
    if (words <= s.plane_words) return CADR_OK;
    // Passes still in flight may use the old area.
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "scratch: synchronize");
    if (s.planes) cudaFree(s.planes);
    s.planes = nullptr;
    s.plane_words = 0;
    e = cudaMalloc(&s.planes, words * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(e, "scratch: planes");
    s.plane_words = words;
    (void)ctx;
    return CADR_OK;
}

cadr_status scratch_reserve(cadr_context* ctx, Scratch& s, uint64_t tiles)
{
    if (tiles <= s.capacity && s.launches < (1ull << 28)) return CADR_OK;
    cudaError_t e;
    if (tiles > s.capacity) {
        // Passes still in flight may use the old area.
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "scratch: synchronize");
        if (s.tile_state) cudaFree(s.tile_state);
        if (s.ctl) cudaFree(s.ctl);
        s.tile_state = nullptr;
        s.ctl = nullptr;
        const uint64_t cap = std::max<uint64_t>(tiles, 1u << 16);
        e = cudaMalloc(&s.tile_state, cap * sizeof(uint64_t));
        if (e != cudaSuccess) return cuda_fail(e, "scratch: tile states");
        e = cudaMalloc(&s.ctl, sizeof(LookbackCtl));
        if (e != cudaSuccess) return cuda_fail(e, "scratch: control block");
        s.capacity = cap;
    } else {
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "scratch: synchronize");
    }
    // Fresh area, or an epoch that is about to wrap: clear everything.
    e = cudaMemset(s.tile_state, 0, s.capacity * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMemset(s.ctl, 0, sizeof(LookbackCtl));
    if (e != cudaSuccess) return cuda_fail(e, "scratch: clear");
    s.launches = 0;
    (void)ctx;
    return CADR_OK;
}

void scratch_release(Scratch& s)
{
    if (s.tile_state) cudaFree(s.tile_state);
    if (s.ctl) cudaFree(s.ctl);
    if (s.planes) cudaFree(s.planes);
    s = Scratch{};
}

static bool is_pinned(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

cadr_status upload_bytes(cadr_context* ctx, void* dst, const void* src, size_t bytes,
                         cudaStream_t stream)
{
    if (bytes == 0) return CADR_OK;
    if (!dst || !src) return fail(CADR_ERR_INVALID_ARG, "upload: null pointer");
    cudaError_t e;
    if (is_pinned(src)) {
        e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return cuda_fail(e, "upload: copy");
        return CADR_OK;
    }
    // Staged through the pinned ring on the upload stream; the consumer
    // stream waits on an event recorded after the last chunk.
    std::lock_guard<std::mutex> lk(ctx->ring_mu);
    const size_t slot_bytes = ctx->ring_bytes / kRingSlots;
    size_t done = 0;
    while (done < bytes) {
        const int slot = ctx->ring_next;
        ctx->ring_next = (ctx->ring_next + 1) % kRingSlots;
        e = cudaEventSynchronize(ctx->ring_event[slot]);
        if (e != cudaSuccess) return cuda_fail(e, "upload: ring wait");
        const size_t n = std::min(slot_bytes, bytes - done);
        uint8_t* stage = ctx->ring + slot * slot_bytes;
        std::memcpy(stage, static_cast<const uint8_t*>(src) + done, n);
        e = cudaMemcpyAsync(static_cast<uint8_t*>(dst) + done, stage, n, cudaMemcpyHostToDevice,
                            ctx->upload_stream);
        if (e != cudaSuccess) return cuda_fail(e, "upload: copy");
        e = cudaEventRecord(ctx->ring_event[slot], ctx->upload_stream);
        if (e != cudaSuccess) return cuda_fail(e, "upload: record");
        done += n;
    }
    e = cudaEventRecord(ctx->upload_done, ctx->upload_stream);
    if (e == cudaSuccess && stream != ctx->upload_stream) e = cudaStreamWaitEvent(stream, ctx->upload_done, 0);
    if (e != cudaSuccess) return cuda_fail(e, "upload: hand-over");
    return CADR_OK;
}

cudaStream_t pick_stream(cadr_context* ctx, cadr_stream s)
{
    return s ? static_cast<cudaStream_t>(s) : ctx->stream;
}

}  // namespace cadr

// ---------------------------------------------------------------------------
extern "C" {

CADR_API int cadr_abi_version(void) { return 1; }

CADR_API uint32_t cadr_build_flags(void)
{
#ifdef CADR_BOUNDS_CHECK
    return CADR_BUILD_BOUNDS_CHECK;
#else
    return 0u;
#endif
}

CADR_API const char* cadr_status_string(cadr_status s)
{
    switch (s) {
    case CADR_OK: return "ok";
    case CADR_ERR_INVALID_ARG: return "invalid argument";
    case CADR_ERR_OUT_OF_MEMORY: return "out of memory";
    case CADR_ERR_TIMEOUT: return "timeout";
    case CADR_ERR_CUDA: return "CUDA error";
    case CADR_ERR_DEVICE: return "device error";
    case CADR_ERR_NOT_READY: return "not ready";
    case CADR_ERR_REJECTED: return "rejected";
    }
    return "unknown status";
}

CADR_API const char* cadr_last_error(void) { return g_last_error.c_str(); }

CADR_API cadr_status cadr_context_create(int device, cadr_context** out)
{
    if (!out) return fail(CADR_ERR_INVALID_ARG, "context_create: null out");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "context_create: no CUDA device");
    if (device < 0 || device >= count) return fail(CADR_ERR_INVALID_ARG, "context_create: bad device %d", device);
    DeviceGuard dg(device);
    e = dg.error();
    if (e != cudaSuccess) return cuda_fail(e, "context_create: set device");
    auto* ctx = new cadr_context();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    // The pass's scattered reads are 4 to 16 bytes wide (handle-table
    // entries, MatrixList headers, parent matrices, LOD entries): DRAM
    // fetches of 32-byte sectors move the fewest unused bytes.  A hint of
    // this process's context, given back when the context is destroyed.
    if (cudaDeviceGetLimit(&ctx->prev_l2_fetch, cudaLimitMaxL2FetchGranularity) == cudaSuccess &&
        cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, kL2FetchBytes) == cudaSuccess)
        ctx->l2_fetch_set = true;
    else
        cudaGetLastError();
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->upload_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->pass_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->shard_counted, cudaEventDisableTiming);
    for (int i = 0; i < kRingSlots && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ctx->ring_event[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->ring), ctx->ring_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_error), sizeof(uint32_t), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->d_error), ctx->h_error, 0);
    if (e != cudaSuccess) {
        cadr_context_destroy(ctx);
        return cuda_fail(e, "context_create");
    }
    *ctx->h_error = 0;
    cadr_status st = scratch_reserve(ctx, ctx->scratch, 1u << 16);
    if (st != CADR_OK) {
        cadr_context_destroy(ctx);
        return st;
    }
    *out = ctx;
    return CADR_OK;
}

CADR_API cadr_status cadr_context_destroy(cadr_context* ctx)
{
    if (!ctx) return CADR_OK;
    DeviceGuard dg(ctx->device);
    cudaDeviceSynchronize();
    destroy_batched_state(ctx);
    if (ctx->l2_fetch_set) cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, ctx->prev_l2_fetch);
    scratch_release(ctx->scratch);
    scratch_release(ctx->shard_scratch);
    for (int f = 0; f < cadr_context::kTsFrames; f++)
        for (int k = 0; k < 4; k++)
            if (ctx->ts_ev[f][k]) cudaEventDestroy(ctx->ts_ev[f][k]);
    for (int f = 0; f < cadr_context::kFrames; f++) {
        for (int k = 0; k < 4; k++)
            if (ctx->frame_ev[f][k]) cudaEventDestroy(ctx->frame_ev[f][k]);
        for (int k = 0; k < CADR_MAX_LEVELS; k++)
            if (ctx->level_ev[f][k]) cudaEventDestroy(ctx->level_ev[f][k]);
    }
    if (ctx->ring) cudaFreeHost(ctx->ring);
    if (ctx->h_error) cudaFreeHost(ctx->h_error);
    for (int i = 0; i < kRingSlots; i++)
        if (ctx->ring_event[i]) cudaEventDestroy(ctx->ring_event[i]);
    if (ctx->upload_done) cudaEventDestroy(ctx->upload_done);
    if (ctx->pass_done) cudaEventDestroy(ctx->pass_done);
    if (ctx->shard_counted) cudaEventDestroy(ctx->shard_counted);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->upload_stream) cudaStreamDestroy(ctx->upload_stream);
    delete ctx;
    return CADR_OK;
}

CADR_API cadr_stream cadr_context_stream(cadr_context* ctx) { return ctx ? ctx->stream : nullptr; }
CADR_API cadr_stream cadr_context_upload_stream(cadr_context* ctx) { return ctx ? ctx->upload_stream : nullptr; }

CADR_API cadr_status cadr_context_set_spin_limit_ns(cadr_context* ctx, uint64_t ns)
{
    if (!ctx || ns == 0) return fail(CADR_ERR_INVALID_ARG, "set_spin_limit: bad argument");
    ctx->spin_limit_ns = ns;
    return CADR_OK;
}

CADR_API cadr_status cadr_context_synchronize(cadr_context* ctx)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "synchronize: null context");
    DeviceGuard dg(ctx->device);
    cudaError_t e = cudaStreamSynchronize(ctx->upload_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "synchronize");
    return CADR_OK;
}

CADR_API uint64_t cadr_context_launch_count(cadr_context* ctx) { return ctx ? ctx->launches.load() : 0; }

CADR_API cadr_status cadr_context_check_device_error(cadr_context* ctx, uint32_t* error_bits)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "check_device_error: null context");
    DeviceGuard dg(ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "check_device_error: synchronize");
    const uint32_t bits = *reinterpret_cast<volatile uint32_t*>(ctx->h_error);
    *ctx->h_error = 0;
    if (error_bits) *error_bits = bits;
    if (bits & CADR_DEVERR_LOOKBACK_TIMEOUT)
        return fail(CADR_ERR_TIMEOUT, "a lookback wait exceeded the spin limit (bits 0x%x)", bits);
    if (bits & CADR_DEVERR_MBARRIER_TIMEOUT)
        return fail(CADR_ERR_TIMEOUT, "an mbarrier wait exceeded the spin limit (bits 0x%x)", bits);
    if (bits) return fail(CADR_ERR_DEVICE, "kernel reported error bits 0x%x", bits);
    return CADR_OK;
}

CADR_API cadr_status cadr_context_set_collect_frame_info(cadr_context* ctx, int on)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "set_collect_frame_info: null context");
    DeviceGuard dg(ctx->device);
    if (on && !ctx->frame_ev[0][0]) {
        for (int f = 0; f < cadr_context::kFrames; f++) {
            for (int k = 0; k < 4; k++) {
                cudaError_t e = cudaEventCreate(&ctx->frame_ev[f][k]);
                if (e != cudaSuccess) return cuda_fail(e, "set_collect_frame_info: events");
            }
            for (int k = 1; k < CADR_MAX_LEVELS; k++) {
                cudaError_t e = cudaEventCreate(&ctx->level_ev[f][k]);
                if (e != cudaSuccess) return cuda_fail(e, "set_collect_frame_info: level events");
            }
        }
    }
    ctx->collect_frames = on != 0;
    ctx->frame_tail = ctx->frame_head;
    return CADR_OK;
}

CADR_API cadr_status cadr_context_get_frame_infos(cadr_context* ctx, cadr_frame_info* out, uint32_t max_frames,
                                                  uint32_t* num_frames)
{
    if (!ctx || !num_frames || (!out && max_frames)) return fail(CADR_ERR_INVALID_ARG, "get_frame_infos: bad argument");
    DeviceGuard dg(ctx->device);
    uint32_t k = 0;
    while (k < max_frames && ctx->frame_tail < ctx->frame_head) {
        const uint64_t f = ctx->frame_tail % cadr_context::kFrames;
        cudaEvent_t* ev = ctx->frame_ev[f];
        cudaEvent_t* lv = ctx->level_ev[f];
        cudaError_t e = cudaEventSynchronize(ev[3]);
        if (e != cudaSuccess) return cuda_fail(e, "get_frame_infos: wait");
        cadr_frame_info& fi = out[k++];
        fi = cadr_frame_info{};
        fi.frame = ctx->frame_tail;
        cudaEventElapsedTime(&fi.propagate_ms, ev[0], ev[1]);
        cudaEventElapsedTime(&fi.leaf_ms, ev[1], ev[3]);
        cudaEventElapsedTime(&fi.total_ms, ev[0], ev[3]);
        cudaEventElapsedTime(&fi.stream_ms, ev[1], ev[2]);
        fi.num_levels = ctx->frame_levels[f];
        for (uint32_t l = 1; l < fi.num_levels; l++)
            cudaEventElapsedTime(&fi.level_ms[l], l == 1 ? ev[0] : lv[l - 1], lv[l]);
        ctx->frame_tail++;
    }
    *num_frames = k;
    return CADR_OK;
}

CADR_API cadr_status cadr_context_record_timestamp(cadr_context* ctx, uint64_t frame, uint32_t index,
                                                  cadr_stream stream)
{
    if (!ctx || index > 3) return fail(CADR_ERR_INVALID_ARG, "record_timestamp: bad argument");
    DeviceGuard dg(ctx->device);
    const int f = (int)(frame % cadr_context::kTsFrames);
    if (!ctx->ts_ev[f][index]) {
        cudaError_t e = cudaEventCreate(&ctx->ts_ev[f][index]);
        if (e != cudaSuccess) return cuda_fail(e, "record_timestamp: event");
    }
    if (ctx->ts_frame[f] != frame) {
        ctx->ts_frame[f] = frame;
        ctx->ts_mask[f] = 0;
    }
    cudaError_t e = cudaEventRecord(ctx->ts_ev[f][index], stream ? (cudaStream_t)stream : ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "record_timestamp: record");
    ctx->ts_mask[f] |= 1u << index;
    return CADR_OK;
}

CADR_API cadr_status cadr_context_read_timestamps(cadr_context* ctx, uint64_t frame, uint64_t* out_ns)
{
    if (!ctx || !out_ns) return fail(CADR_ERR_INVALID_ARG, "read_timestamps: null argument");
    const int f = (int)(frame % cadr_context::kTsFrames);
    if (ctx->ts_frame[f] != frame || ctx->ts_mask[f] != 0xFu)
        return fail(CADR_ERR_INVALID_ARG, "read_timestamps: frame %llu does not have its four timestamps",
                    (unsigned long long)frame);
    DeviceGuard dg(ctx->device);
    cudaError_t e = cudaEventSynchronize(ctx->ts_ev[f][3]);
    if (e != cudaSuccess) return cuda_fail(e, "read_timestamps: wait");
    out_ns[0] = 0;
    for (int k = 1; k < 4; k++) {
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, ctx->ts_ev[f][0], ctx->ts_ev[f][k]);
        if (e != cudaSuccess) return cuda_fail(e, "read_timestamps: elapsed");
        out_ns[k] = (uint64_t)((double)ms * 1e6 + 0.5);
    }
    return CADR_OK;
}

CADR_API cadr_status cadr_debug_set_fault(cadr_context* ctx, uint32_t fault)
{
    if (!ctx || fault > CADR_FAULT_SERVER_LAUNCH) return fail(CADR_ERR_INVALID_ARG, "debug_set_fault: bad argument");
    __atomic_store_n(&ctx->fault, fault, __ATOMIC_RELAXED);  // the server's scheduler thread reads it
    return CADR_OK;
}

CADR_API cadr_status cadr_device_alloc(cadr_context* ctx, size_t bytes, void** out)
{
    if (!ctx || !out) return fail(CADR_ERR_INVALID_ARG, "device_alloc: null argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    if (bytes == 0) return CADR_OK;
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "device_alloc");
    return CADR_OK;
}

CADR_API cadr_status cadr_device_free(cadr_context* ctx, void* ptr)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "device_free: null context");
    DeviceGuard dg(ctx->device);
    if (!ptr) return CADR_OK;
    cudaError_t e = cudaFree(ptr);
    if (e != cudaSuccess) return cuda_fail(e, "device_free");
    return CADR_OK;
}

CADR_API cadr_status cadr_host_alloc_pinned(size_t bytes, void** out)
{
    if (!out) return fail(CADR_ERR_INVALID_ARG, "host_alloc_pinned: null out");
    cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(e, "host_alloc_pinned");
    return CADR_OK;
}

CADR_API cadr_status cadr_host_free_pinned(void* ptr)
{
    if (!ptr) return CADR_OK;
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return cuda_fail(e, "host_free_pinned");
    return CADR_OK;
}

CADR_API cadr_status cadr_upload(cadr_context* ctx, void* dst_device, const void* src_host, size_t bytes,
                                 cadr_stream stream)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "upload: null context");
    DeviceGuard dg(ctx->device);
    return upload_bytes(ctx, dst_device, src_host, bytes, pick_stream(ctx, stream));
}

CADR_API cadr_status cadr_download(cadr_context* ctx, void* dst_host, const void* src_device, size_t bytes,
                                   cadr_stream stream)
{
    if (!ctx || (!dst_host && bytes) || (!src_device && bytes)) return fail(CADR_ERR_INVALID_ARG, "download: bad argument");
    DeviceGuard dg(ctx->device);
    if (bytes == 0) return CADR_OK;
    cudaError_t e = cudaMemcpyAsync(dst_host, src_device, bytes, cudaMemcpyDeviceToHost, pick_stream(ctx, stream));
    if (e != cudaSuccess) return cuda_fail(e, "download");
    return CADR_OK;
}

CADR_API cadr_status cadr_download_commands(cadr_context* ctx, cadr_draw_indexed_cmd* host_cmds,
                                            const cadr_draw_indexed_cmd* device_cmds, const uint32_t* host_counts,
                                            const uint32_t* host_offsets, uint32_t num_state_sets, uint64_t* bytes,
                                            cadr_stream stream)
{
    if (!ctx || !host_counts || !host_offsets || (num_state_sets && (!host_cmds || !device_cmds)))
        return fail(CADR_ERR_INVALID_ARG, "download_commands: null argument");
    DeviceGuard dg(ctx->device);
    for (uint32_t k = 0; k < num_state_sets; k++)
        if (host_offsets[k + 1] < host_offsets[k] || host_counts[k] > host_offsets[k + 1] - host_offsets[k])
            return fail(CADR_ERR_INVALID_ARG, "download_commands: count %u exceeds StateSet region %u", host_counts[k], k);
    cudaStream_t st = pick_stream(ctx, stream);
    uint64_t total = 0;
    uint32_t k = 0;
    while (k < num_state_sets) {
        if (!host_counts[k]) {
            k++;
            continue;
        }
        // Regions whose valid parts touch (every region before the last one
        // of the run full) go in one copy.
        const uint32_t first = host_offsets[k];
        uint32_t end = first + host_counts[k];
        while (k + 1 < num_state_sets && end == host_offsets[k + 1] && host_counts[k + 1]) {
            k++;
            end = host_offsets[k] + host_counts[k];
        }
        const size_t nbytes = (size_t)(end - first) * sizeof(cadr_draw_indexed_cmd);
        const cudaError_t e = cudaMemcpyAsync(host_cmds + first, device_cmds + first, nbytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_fail(e, "download_commands");
        total += nbytes;
        k++;
    }
    if (bytes) *bytes = total;
    return CADR_OK;
}

CADR_API cadr_status cadr_stream_synchronize(cadr_stream stream)
{
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "stream_synchronize");
    return CADR_OK;
}

// ---------------------------------------------------------------------------
// Tier A.

CADR_API cadr_status cadr_process_drawables(cadr_context* ctx, uint32_t handle_level, const void* handle_table,
                                            const cadr_drawable_gpu_data* drawables, uint64_t num_drawables,
                                            cadr_draw_indirect_cmd* indirect, cadr_drawable_pointers* pointers,
                                            cadr_stream stream)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "process_drawables: null context");
    DeviceGuard dg(ctx->device);
    if (handle_level < 1 || handle_level > 3)
        return fail(CADR_ERR_INVALID_ARG, "process_drawables: handle level %u not in 1..3", handle_level);
    if (num_drawables == 0) return CADR_OK;
    if (!handle_table || !drawables || !indirect || !pointers)
        return fail(CADR_ERR_INVALID_ARG, "process_drawables: null buffer");
    if ((reinterpret_cast<uintptr_t>(drawables) | reinterpret_cast<uintptr_t>(indirect) |
         reinterpret_cast<uintptr_t>(pointers)) & 15u)
        return fail(CADR_ERR_INVALID_ARG, "process_drawables: buffers must be 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(handle_table) & 7u)
        return fail(CADR_ERR_INVALID_ARG, "process_drawables: handle table must be 8-byte aligned");
    // The reference dispatches at most 32768*32768 workgroups (Renderer.cpp:688).
    if (num_drawables >= (1ull << 30))
        return fail(CADR_ERR_INVALID_ARG, "process_drawables: limit of 1Gi drawables reached");
    cudaError_t e = launch_process_drawables(handle_level, static_cast<const uint64_t*>(handle_table), drawables,
                                             num_drawables, indirect, pointers, pick_stream(ctx, stream));
    if (e != cudaSuccess) return cuda_fail(e, "process_drawables: launch");
    ctx->launches++;
    return CADR_OK;
}

}  // extern "C"
