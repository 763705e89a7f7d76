// pack.cu - device-resident StateSet packing of the Tier A records.
//
// The reference packs on the host every frame: StateSet::prepareRecording
// counts the drawables of every subtree (src/CadR/StateSet.cpp:180-195) and
// StateSet::recordToCommandBuffer walks the StateSets depth-first, copying
// each one's DrawableGpuData list, in list order, into the staging buffer
// at drawableCounter and drawing it with one cmdDrawIndirect
// (StateSet.cpp:198-268); Renderer::recordDrawableProcessing then uploads
// the staging buffer (Renderer.cpp:635-644).  For 16.8 M drawables that is
// 805 MB of host memcpy and PCIe/C2C traffic per frame.
//
// Here the records stay on the device in a pool indexed by slot.  A layout
// gives every slot its StateSet and its position in that StateSet's list,
// and the StateSets' depth-first order; from it the device derives each
// StateSet's region (the drawableCounter at which the reference copies it)
// and the slot <-> packed-position maps.  A repack gathers the pool into
// the packed array; a frame whose records changed patches only those rows,
// in the pool and in the packed array.
#include <cuda_runtime.h>

#include <algorithm>

#include "capi_internal.h"
#include "handles.cuh"

using namespace cadr;

struct cadr_pack {
    cadr_context* ctx = nullptr;
    uint32_t capacity = 0;
    uint32_t num_slots = 0;
    uint32_t num_state_sets = 0;
    uint4* pool = nullptr;       // capacity records (3 uint4 each), by slot
    uint4* packed = nullptr;     // capacity records, depth-first order
    uint32_t* pos_of_slot = nullptr;
    uint32_t* slot_of_pos = nullptr;
    uint32_t* set_of_slot = nullptr;   // layout input
    uint32_t* index_of_slot = nullptr; // layout input
    uint32_t* sets = nullptr;          // 4 arrays of set_cap words: dfs order, rank, count, start
    uint32_t* offsets = nullptr;       // set_cap + 1 words: region offsets in depth-first order
    uint32_t set_cap = 0;
    uint32_t* patch_slots = nullptr;   // patch staging
    uint4* patch_records = nullptr;
    uint32_t patch_cap = 0;
};

namespace cadr {
namespace {

constexpr uint32_t kNoSlot = 0xffffffffu;
constexpr int kPackThreads = 256;

// Per-StateSet drawable counts and the depth-first rank of every StateSet
// (rank[dfs[j]] = j; a repeated StateSet id in dfs is an error).  With at
// most kSmemBins StateSets each CTA counts into shared memory and adds its
// non-zero bins once: a few StateSets holding millions of drawables would
// otherwise serialise on a few global counters.
constexpr uint32_t kSmemBins = 4096;

__global__ void __launch_bounds__(kPackThreads) pack_count_kernel(const uint32_t* __restrict__ set_of_slot, uint32_t n,
                                                                  uint32_t S, const uint32_t* __restrict__ dfs,
                                                                  uint32_t* __restrict__ rank,
                                                                  uint32_t* __restrict__ count, uint32_t* error)
{
    __shared__ uint32_t bins[kSmemBins];
    const bool local = S <= kSmemBins;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (local) {
        for (uint32_t b = threadIdx.x; b < S; b += blockDim.x) bins[b] = 0;
        __syncthreads();
    }
    if (k < S) {
        const uint32_t s = dfs[k];
        if (s >= S || atomicExch(&rank[s], k) != kNoSlot) atomicOr(error, CADR_DEVERR_BAD_INDEX);
    }
    if (k < n) {
        const uint32_t s = set_of_slot[k];
        if (s >= S)
            atomicOr(error, CADR_DEVERR_BAD_INDEX);
        else if (local)
            atomicAdd(&bins[s], 1u);
        else
            atomicAdd(&count[s], 1u);
    }
    if (local) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < S; b += blockDim.x)
            if (bins[b]) atomicAdd(&count[b], bins[b]);
    }
}

// One CTA: offsets[j] = drawables of the StateSets before dfs[j] in
// depth-first order (the reference's drawableCounter), offsets[S] = total;
// start[s] = offsets[rank[s]].
__global__ void __launch_bounds__(1024) pack_offsets_kernel(const uint32_t* __restrict__ dfs,
                                                             const uint32_t* __restrict__ count, uint32_t S,
                                                             uint32_t* __restrict__ offsets,
                                                             uint32_t* __restrict__ start)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_run;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    if (t == 0) s_run = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < S; c0 += blockDim.x) {
        const uint32_t j = c0 + t;
        const uint32_t s = j < S ? dfs[j] : 0u;
        const uint32_t v = (j < S && s < S) ? count[s] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, incl, o);
            if (lane >= (uint32_t)o) incl += u;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t nw = blockDim.x / 32u;
            uint32_t w = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(~0u, w, o);
                if (lane >= (uint32_t)o) w += u;
            }
            s_warp[lane] = w;  // inclusive over warps 0..lane
        }
        __syncthreads();
        const uint32_t excl = s_run + (warp ? s_warp[warp - 1] : 0u) + incl - v;
        if (j < S) {
            offsets[j] = excl;
            if (s < S) start[s] = excl;
        }
        __syncthreads();
        if (t == blockDim.x - 1) s_run = excl + v;
        __syncthreads();
    }
    if (t == 0) offsets[S] = s_run;
}

// Packed position of every slot: start of its StateSet + its list index.
// A list index outside its StateSet's list, or a position claimed twice,
// is an error (then some position stays unclaimed).
__global__ void pack_place_kernel(const uint32_t* __restrict__ set_of_slot, const uint32_t* __restrict__ index_of_slot,
                                  uint32_t n, uint32_t S, const uint32_t* __restrict__ count,
                                  const uint32_t* __restrict__ start, uint32_t* __restrict__ pos_of_slot,
                                  uint32_t* __restrict__ slot_of_pos, uint32_t* error)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t s = set_of_slot[k], li = index_of_slot[k];
    if (s >= S || li >= count[s]) {
        atomicOr(error, CADR_DEVERR_BAD_INDEX);
        pos_of_slot[k] = kNoSlot;
        return;
    }
    const uint32_t p = start[s] + li;
    if (!CADR_CHECKED(p < n, error)) {
        pos_of_slot[k] = kNoSlot;
        return;
    }
    pos_of_slot[k] = p;
    if (atomicExch(&slot_of_pos[p], k) != kNoSlot) atomicOr(error, CADR_DEVERR_BAD_INDEX);
}

// packed[p] = pool[slot_of_pos[p]]: 48-byte records as three 16-byte
// words, consecutive threads on consecutive words of the packed array.
__global__ void pack_gather_kernel(const uint4* __restrict__ pool, const uint32_t* __restrict__ slot_of_pos,
                                   uint32_t n, uint4* __restrict__ packed)
{
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= 3ull * n) return;
    const uint32_t p = (uint32_t)(w / 3), part = (uint32_t)(w % 3);
    const uint32_t k = __ldg(slot_of_pos + p);
    if (k == kNoSlot) return;  // only after a layout error
    packed[w] = __ldg(pool + 3ull * k + part);
}

// Dirty rows: pool[slots[j]] = packed[pos(slots[j])] = records[j].
__global__ void pack_patch_kernel(const uint32_t* __restrict__ slots, const uint4* __restrict__ records,
                                  uint32_t count, uint32_t n, const uint32_t* __restrict__ pos_of_slot,
                                  uint4* __restrict__ pool, uint4* __restrict__ packed, uint32_t* error)
{
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= 3ull * count) return;
    const uint32_t j = (uint32_t)(w / 3), part = (uint32_t)(w % 3);
    const uint32_t k = __ldg(slots + j);
    if (k >= n) {
        if (part == 0) atomicOr(error, CADR_DEVERR_BAD_INDEX);
        return;
    }
    const uint4 r = __ldg(records + w);
    pool[3ull * k + part] = r;
    const uint32_t p = __ldg(pos_of_slot + k);
    if (p != kNoSlot) packed[3ull * p + part] = r;
}

// Tier A straight from the pool: slot k's record is resolved and its
// indirect command and pointers are written at its packed position, for
// the positions below n_draw.  Slots come in the order their drawables
// were created, which is also the order of their MatrixList and
// drawable-data handles, so the handle-table reads of a warp fall on
// neighbouring entries; the outputs are scattered instead.  A slot outside
// the drawn positions is not read at all.
template <int LEVEL>
__global__ void __launch_bounds__(256) pack_process_kernel(const uint64_t* __restrict__ root,
                                                           const ulonglong2* __restrict__ pool,
                                                           const uint32_t* __restrict__ pos_of_slot, uint32_t n,
                                                           uint32_t n_draw, uint4* __restrict__ indirect,
                                                           ulonglong2* __restrict__ pointers)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t p = __ldg(pos_of_slot + k);
    if (p >= n_draw) return;  // also kNoSlot
    const ulonglong2* d = pool + 3ull * k;
    uint4 ind;
    ulonglong2 p0, p1;
    resolve_record<LEVEL>(root, __ldg(d), __ldg(d + 1), __ldg(d + 2), ind, p0, p1);
    indirect[p] = ind;
    pointers[2ull * p] = p0;
    pointers[2ull * p + 1] = p1;
}

uint32_t blocks(uint64_t items) { return (uint32_t)((items + kPackThreads - 1) / kPackThreads); }

void release(cadr_pack* pk)
{
    cudaFree(pk->pool);
    cudaFree(pk->packed);
    cudaFree(pk->pos_of_slot);
    cudaFree(pk->slot_of_pos);
    cudaFree(pk->set_of_slot);
    cudaFree(pk->index_of_slot);
    cudaFree(pk->sets);
    cudaFree(pk->offsets);
    cudaFree(pk->patch_slots);
    cudaFree(pk->patch_records);
}

}  // namespace
}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_pack_create(cadr_context* ctx, uint32_t capacity, cadr_pack** out)
{
    if (!ctx || !out) return fail(CADR_ERR_INVALID_ARG, "pack_create: null argument");
    DeviceGuard dg(ctx->device);
    *out = nullptr;
    cudaError_t e = dg.error();
    if (e != cudaSuccess) return cuda_fail(e, "pack_create: set device");
    auto* pk = new cadr_pack();
    pk->ctx = ctx;
    pk->capacity = capacity;
    const size_t rec = (size_t)std::max<uint32_t>(capacity, 1u) * sizeof(cadr_drawable_gpu_data);
    const size_t word = (size_t)std::max<uint32_t>(capacity, 1u) * sizeof(uint32_t);
    e = cudaMalloc(&pk->pool, rec);
    if (e == cudaSuccess) e = cudaMalloc(&pk->packed, rec);
    if (e == cudaSuccess) e = cudaMalloc(&pk->pos_of_slot, word);
    if (e == cudaSuccess) e = cudaMalloc(&pk->slot_of_pos, word);
    if (e == cudaSuccess) e = cudaMalloc(&pk->set_of_slot, word);
    if (e == cudaSuccess) e = cudaMalloc(&pk->index_of_slot, word);
    if (e != cudaSuccess) {
        release(pk);
        delete pk;
        return cuda_fail(e, "pack_create: allocate");
    }
    *out = pk;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_destroy(cadr_pack* pack)
{
    if (!pack) return CADR_OK;
    DeviceGuard dg(pack->ctx->device);
    cudaDeviceSynchronize();
    release(pack);
    delete pack;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_set_layout(cadr_pack* pk, uint32_t num_slots, uint32_t num_state_sets,
                                          const uint32_t* dfs_order, const uint32_t* state_set_of_slot,
                                          const uint32_t* list_index_of_slot, cadr_stream stream)
{
    if (!pk || !dfs_order || (num_slots && (!state_set_of_slot || !list_index_of_slot)))
        return fail(CADR_ERR_INVALID_ARG, "pack_set_layout: null argument");
    DeviceGuard dg(pk->ctx->device);
    if (num_slots > pk->capacity)
        return fail(CADR_ERR_INVALID_ARG, "pack_set_layout: %u slots exceed the capacity %u", num_slots,
                    pk->capacity);
    if (num_state_sets == 0) return fail(CADR_ERR_INVALID_ARG, "pack_set_layout: no StateSet");
    cadr_context* ctx = pk->ctx;
    cudaStream_t s = pick_stream(ctx, stream);
    cudaError_t e;
    if (num_state_sets > pk->set_cap) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "pack_set_layout: synchronize");
        cudaFree(pk->sets);
        cudaFree(pk->offsets);
        pk->sets = nullptr;
        pk->offsets = nullptr;
        pk->set_cap = 0;
        e = cudaMalloc(&pk->sets, (size_t)num_state_sets * 4 * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&pk->offsets, ((size_t)num_state_sets + 1) * sizeof(uint32_t));
        if (e != cudaSuccess) return cuda_fail(e, "pack_set_layout: allocate");
        pk->set_cap = num_state_sets;
    }
    const uint32_t S = num_state_sets, n = num_slots;
    uint32_t* dfs = pk->sets;
    uint32_t* rank = pk->sets + S;
    uint32_t* count = pk->sets + 2 * (size_t)S;
    uint32_t* start = pk->sets + 3 * (size_t)S;
    cadr_status st = upload_bytes(ctx, dfs, dfs_order, (size_t)S * 4, s);
    if (st == CADR_OK) st = upload_bytes(ctx, pk->set_of_slot, state_set_of_slot, (size_t)n * 4, s);
    if (st == CADR_OK) st = upload_bytes(ctx, pk->index_of_slot, list_index_of_slot, (size_t)n * 4, s);
    if (st != CADR_OK) return st;
    e = cudaMemsetAsync(rank, 0xff, (size_t)S * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, (size_t)S * 4, s);
    if (e == cudaSuccess && n) e = cudaMemsetAsync(pk->slot_of_pos, 0xff, (size_t)n * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "pack_set_layout: clear");
    pack_count_kernel<<<blocks(std::max(n, S)), kPackThreads, 0, s>>>(pk->set_of_slot, n, S, dfs, rank, count,
                                                                      ctx->d_error);
    pack_offsets_kernel<<<1, 1024, 0, s>>>(dfs, count, S, pk->offsets, start);
    if (n)
        pack_place_kernel<<<blocks(n), kPackThreads, 0, s>>>(pk->set_of_slot, pk->index_of_slot, n, S, count,
                                                              start, pk->pos_of_slot, pk->slot_of_pos,
                                                              ctx->d_error);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "pack_set_layout: launch");
    ctx->launches += n ? 3 : 2;
    pk->num_slots = n;
    pk->num_state_sets = S;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_upload(cadr_pack* pk, const cadr_drawable_gpu_data* records, uint32_t first,
                                      uint32_t count, cadr_stream stream)
{
    if (!pk || (count && !records)) return fail(CADR_ERR_INVALID_ARG, "pack_upload: null argument");
    DeviceGuard dg(pk->ctx->device);
    if ((uint64_t)first + count > pk->capacity)
        return fail(CADR_ERR_INVALID_ARG, "pack_upload: slots [%u, %llu) exceed the capacity %u", first,
                    (unsigned long long)first + count, pk->capacity);
    return upload_bytes(pk->ctx, pk->pool + 3ull * first, records, (size_t)count * sizeof(cadr_drawable_gpu_data),
                        pick_stream(pk->ctx, stream));
}

CADR_API cadr_status cadr_pack_repack(cadr_pack* pk, cadr_stream stream)
{
    if (!pk) return fail(CADR_ERR_INVALID_ARG, "pack_repack: null pack");
    DeviceGuard dg(pk->ctx->device);
    if (pk->num_slots == 0) return CADR_OK;
    cudaStream_t s = pick_stream(pk->ctx, stream);
    pack_gather_kernel<<<blocks(3ull * pk->num_slots), kPackThreads, 0, s>>>(pk->pool, pk->slot_of_pos, pk->num_slots,
                                                                             pk->packed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "pack_repack: launch");
    pk->ctx->launches++;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_patch(cadr_pack* pk, const uint32_t* slots, const cadr_drawable_gpu_data* records,
                                     uint32_t count, cadr_stream stream)
{
    if (!pk || (count && (!slots || !records))) return fail(CADR_ERR_INVALID_ARG, "pack_patch: null argument");
    DeviceGuard dg(pk->ctx->device);
    if (count == 0) return CADR_OK;
    cadr_context* ctx = pk->ctx;
    cudaStream_t s = pick_stream(ctx, stream);
    cudaError_t e;
    if (count > pk->patch_cap) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "pack_patch: synchronize");
        cudaFree(pk->patch_slots);
        cudaFree(pk->patch_records);
        pk->patch_slots = nullptr;
        pk->patch_records = nullptr;
        pk->patch_cap = 0;
        const uint32_t cap = std::max<uint32_t>(count, 1u << 16);
        e = cudaMalloc(&pk->patch_slots, (size_t)cap * 4);
        if (e == cudaSuccess) e = cudaMalloc(&pk->patch_records, (size_t)cap * sizeof(cadr_drawable_gpu_data));
        if (e != cudaSuccess) return cuda_fail(e, "pack_patch: allocate");
        pk->patch_cap = cap;
    }
    cadr_status st = upload_bytes(ctx, pk->patch_slots, slots, (size_t)count * 4, s);
    if (st == CADR_OK)
        st = upload_bytes(ctx, pk->patch_records, records, (size_t)count * sizeof(cadr_drawable_gpu_data), s);
    if (st != CADR_OK) return st;
    pack_patch_kernel<<<blocks(3ull * count), kPackThreads, 0, s>>>(pk->patch_slots, pk->patch_records, count,
                                                                    pk->num_slots, pk->pos_of_slot, pk->pool,
                                                                    pk->packed, ctx->d_error);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "pack_patch: launch");
    ctx->launches++;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_process_drawables(cadr_pack* pk, uint32_t handle_level, const void* handle_table,
                                                 uint32_t num_draw_records, cadr_draw_indirect_cmd* indirect,
                                                 cadr_drawable_pointers* pointers, cadr_stream stream)
{
    if (!pk || (num_draw_records && (!handle_table || !indirect || !pointers)))
        return fail(CADR_ERR_INVALID_ARG, "pack_process_drawables: null argument");
    DeviceGuard dg(pk->ctx->device);
    if (handle_level < 1 || handle_level > 3)
        return fail(CADR_ERR_INVALID_ARG, "pack_process_drawables: handle level %u", handle_level);
    if (num_draw_records > pk->num_slots)
        return fail(CADR_ERR_INVALID_ARG, "pack_process_drawables: %u records drawn, %u in the layout",
                    num_draw_records, pk->num_slots);
    if ((reinterpret_cast<uintptr_t>(handle_table) | reinterpret_cast<uintptr_t>(indirect) |
         reinterpret_cast<uintptr_t>(pointers)) % 16)
        return fail(CADR_ERR_INVALID_ARG, "pack_process_drawables: misaligned buffer");
    if (num_draw_records == 0) return CADR_OK;
    cudaStream_t s = pick_stream(pk->ctx, stream);
    auto root = static_cast<const uint64_t*>(handle_table);
    auto pool = reinterpret_cast<const ulonglong2*>(pk->pool);
    auto ind = reinterpret_cast<uint4*>(indirect);
    auto ptr = reinterpret_cast<ulonglong2*>(pointers);
    const uint32_t grid = blocks(pk->num_slots);
    switch (handle_level) {
    case 1: pack_process_kernel<1><<<grid, 256, 0, s>>>(root, pool, pk->pos_of_slot, pk->num_slots, num_draw_records, ind, ptr); break;
    case 2: pack_process_kernel<2><<<grid, 256, 0, s>>>(root, pool, pk->pos_of_slot, pk->num_slots, num_draw_records, ind, ptr); break;
    default: pack_process_kernel<3><<<grid, 256, 0, s>>>(root, pool, pk->pos_of_slot, pk->num_slots, num_draw_records, ind, ptr); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "pack_process_drawables: launch");
    pk->ctx->launches++;
    return CADR_OK;
}

CADR_API cadr_status cadr_pack_buffers(cadr_pack* pk, const cadr_drawable_gpu_data** packed,
                                       const uint32_t** region_offsets, uint32_t* num_slots)
{
    if (!pk) return fail(CADR_ERR_INVALID_ARG, "pack_buffers: null pack");
    if (packed) *packed = reinterpret_cast<const cadr_drawable_gpu_data*>(pk->packed);
    if (region_offsets) *region_offsets = pk->offsets;
    if (num_slots) *num_slots = pk->num_slots;
    return CADR_OK;
}

}  // extern "C"
