// batched.cu - the batched form: many (scene, view) pairs culled by one
// persistent launch over (view, tile) work items.
//
// Scenes are propagated once (cadr_scene_propagate with world spheres); each
// view then reads only the 16-byte world sphere and the 4-byte geometry
// index of every drawable.  Work items are numbered view-major and handed
// out by an atomic counter, so the items a tile looks back on were taken
// earlier by resident CTAs.  The arithmetic per (view, drawable) is the
// plain pass's (same classify, same compaction), so outputs are identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "compact.cuh"

namespace cadr {

struct BatchedState {
    ViewJob* d_jobs = nullptr;
    ViewJob* h_jobs = nullptr;  // pinned; read by the graph's copy node
    uint32_t cap = 0;
    cudaEvent_t jobs_free = nullptr;
    bool jobs_pending = false;
    Scratch scratch;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t key_views = 0, key_items = 0, key_grid = 0;
    cadr_tuning key_tuning = {};
    cudaStream_t key_stream = nullptr;
    uint64_t key_limit = 0;
    uint32_t key_fault = 0;
};

namespace {

// StateSet offsets of the current view's scene are staged in shared memory
// up to this many entries (8 KiB).
constexpr uint32_t kBatchedOffsetCap = 2048;

// The job of work item `item`, found by one warp: each round its lanes
// probe 32 evenly spaced jobs and keep the last whose first item is at or
// below `item` (two rounds up to 1,024 jobs).  jobs[0].first_item is 0.
__device__ __forceinline__ uint32_t warp_find_job(const ViewJob* __restrict__ jobs, uint32_t num_jobs, uint32_t item)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lo = 0, hi = num_jobs;  // the job is in [lo, hi); jobs[lo].first_item <= item
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31u) / 32u;
        const uint32_t k = lo + lane * step;
        const uint32_t m = __ballot_sync(~0u, k < hi && __ldg(&jobs[k].first_item) <= item);
        lo += (31u - (uint32_t)__clz(m)) * step;  // lane 0 always holds: bit 0 is set
        hi = min(hi, lo + step);
    }
    return lo;
}

// The persistent kernel.  Per item: warp 0 publishes the item (lane 0
// takes it) and its job (the warp's two-round search) by the first
// barrier; load and classify, barrier; warp 0 scans the tile, publishes
// the tile's aggregate and looks back while the other warps gather their
// LOD entries, barrier; write.  The per-item tile state
// is double-buffered (item k uses sm[k & 1]), so the next item's ballots
// never overwrite what a slower warp still reads in this item's write
// phase, and the first barrier of the next item, which every thread
// reaches only after its writes, guards the job record: three CTA barriers
// per item.  Thread 0 takes the next item while the current one's commands
// are written (the atomic's round trip leaves the critical path), so a CTA
// holds an item it has not started only for one write phase.
// Launch bounds of 1,024 threads per SM cap the kernel at 64 registers:
// at 80 (unbounded) only three 256-thread CTAs fit an SM and the item chain
// of each has fewer neighbours to hide behind; capped, four fit, and C4 ran
// 0.737 -> 0.671 ms (a 24-byte spill at 8 items per thread).  The job
// search by the whole warp (two dependent rounds) and the branch-free
// plane tests of classify() took it to 0.657 ms.
template <int THREADS, int IPT>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batched_kernel(const ViewJob* __restrict__ jobs, uint32_t num_jobs,
                                                         uint32_t total_items, const Scratch s, uint32_t* error,
                                                         uint64_t limit_ns, uint32_t fault)
{
    using T = Tile<THREADS, IPT>;
    __shared__ typename T::Smem sm[2];
    __shared__ __align__(16) ViewJob job;
    __shared__ uint32_t s_item, s_job;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    extern __shared__ uint32_t s_offsets[];
    if (t == 0) {
        const uint32_t ep = load_relaxed_u32(&s.ctl->epoch);
        sm[0].info[1] = ep;
        sm[1].info[1] = ep;
    }
    uint32_t cur = 0, cur_job = 0xffffffffu;
    const uint32_t* off = nullptr;
    uint32_t nxt = 0;
    bool have_next = false;
    for (;;) {
        if (warp == 0) {
            uint32_t it = 0;
            if (lane == 0) it = have_next ? nxt : atomicAdd(&s.ctl->tile_counter, 1u);
            it = __shfl_sync(~0u, it, 0);
            const uint32_t jb = it < total_items ? warp_find_job(jobs, num_jobs, it) : 0u;
            if (lane == 0) {
                s_item = it;
                s_job = jb;
            }
        }
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total_items) break;
        if (s_job != cur_job) {
            cur_job = s_job;
            const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + cur_job);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&job);
            for (int k = t; k < (int)(sizeof(ViewJob) / 4); k += THREADS) dst[k] = __ldg(src + k);
            __syncthreads();
            // published by the __syncthreads() that follows the item loop
            off = stage_offsets(s_offsets, kBatchedOffsetCap, job.offsets, job.num_state_sets);
        }
        typename T::Smem& S = sm[cur];
        const uint32_t n = job.n;
        const uint32_t b = (item - job.first_item) * (uint32_t)T::SIZE;
        // The warp search found the item's job: the item is one of its
        // tiles.  (Reads are clamped and writes check their regions; this
        // reports a wrong job table.)
        if (t == 0)
            (void)CADR_CHECKED(item >= job.first_item && item - job.first_item < max(1u, (n + T::SIZE - 1) / T::SIZE),
                               error);
        uint32_t vis_bits = 0, lod_bits = 0;
        uint32_t geo[IPT];
        float4 wsv[IPT];
        // Every item's inputs in flight together, then the arithmetic.
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const uint32_t i = b + (uint32_t)(j * THREADS + t);
            const uint32_t ic = i < n ? i : 0u;
            wsv[j] = n ? ld_nc_f4(job.world_sphere + ic) : make_float4(0.f, 0.f, 0.f, 0.f);
            geo[j] = n ? ld_nc_u32(job.geometry + ic) : 0u;
        }
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const uint32_t i = b + (uint32_t)(j * THREADS + t);
            bool visible = false, marginal = false;
            uint32_t lod = 0;
            if (i < n)
                classify(job.view, wsv[j], job.num_lods, visible, marginal, lod);
            else
                geo[j] = 0;
            const uint32_t vb = __ballot_sync(~0u, visible);
            const uint32_t mb = __ballot_sync(~0u, marginal);
            const uint32_t word0 = b + (uint32_t)(j * THREADS + warp * kWarp);
            if (lane == 0) {
                S.ballot[j][warp] = vb;
                if (job.marginal && word0 < n) job.marginal[word0 >> 5] = mb;
            }
            vis_bits |= (visible ? 1u : 0u) << j;
            lod_bits |= lod << (2 * j);
        }
        __syncthreads();
        // Warp 0 scans the tile and publishes its aggregate first; the LOD
        // entries are gathered while it waits for its predecessor's prefix.
        if (warp == 0) {
            T::scan_warp0(S, off, job.num_state_sets, b, n);
            if (t == 0) T::publish(S, s.tile_state, item, job.first_item, off, b, fault);
        }
        uint4 ent[IPT];
        T::gather(vis_bits, lod_bits, geo, job.lods, job.num_geometries, job.num_lods, error, ent);
        if (warp == 0) T::resolve(S, s.tile_state, item, job.first_item, limit_ns, error);
        __syncthreads();
        if (t == 0) {
            nxt = atomicAdd(&s.ctl->tile_counter, 1u);
            have_next = true;
        }
        T::write_ent(S, vis_bits, ent, b, n, item == job.first_item, off, job.num_state_sets, job.cmds, job.counts,
                     error);
        cur ^= 1u;
    }
    if (t == 0) finish_pass(s.ctl);
}

// ---------------------------------------------------------------------------
// The three-launch form (tuning form 1): classify, per-view tile scan,
// write, over the same view-major (view, tile) items with tiles of
// kLeafTile drawables, so that each scene's per-tile region-start table
// serves it.  No CTA waits for another: a reduce-then-scan like the plain
// pass, with every view's first tile a scan head.

// Words of one bit-plane of a batch: 64 per item (2,048 drawables), padded
// to 16 bytes.  Three planes (visibility, LOD bits 0 and 1), then one tile
// word per item.
__host__ __device__ constexpr uint64_t batched_plane_stride(uint64_t items) { return (items * 64 + 3) & ~uint64_t(3); }

// Launch 1: one CTA per item classifies its drawables into the planes and
// writes the item's tile word (as the plain pass's stream kernel does from
// its matrices, here from the scene's world spheres).
__global__ void __launch_bounds__(kLeafThreads) batched_classify_kernel(const ViewJob* __restrict__ jobs,
                                                                       uint32_t num_jobs, uint32_t* __restrict__ planes,
                                                                       uint64_t stride)
{
    __shared__ ViewConst s_view;
    __shared__ uint32_t ballot[kLeafIpt][kLeafWarps];
    __shared__ uint32_t s_last_start;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t item = blockIdx.x;
    const ViewJob* J = jobs + warp_find_job(jobs, num_jobs, item);
    const uint32_t n = J->n, num_lods = J->num_lods;
    const uint32_t tile = item - J->first_item;
    const uint32_t b = tile * (uint32_t)kLeafTile;
    if (warp == 0) {
        if (lane < (int)(sizeof(ViewConst) / 16))
            reinterpret_cast<uint4*>(&s_view)[lane] = __ldg(reinterpret_cast<const uint4*>(&J->view) + lane);
        if (lane == 31) s_last_start = n ? __ldg(J->tile_start + tile) : 0u;
    }
    const float4* ws = J->world_sphere;
    uint32_t* marginal = J->marginal;
    float4 wsv[kLeafIpt];
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i = b + (uint32_t)(j * kLeafThreads + t);
        wsv[j] = i < n ? ld_nc_f4(ws + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const uint64_t base = (uint64_t)item * 64;
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
        bool visible = false, mar = false;
        uint32_t lod = 0;
        if (i0 + (uint32_t)lane < n) classify(s_view, wsv[j], num_lods, visible, mar, lod);
        const uint32_t vb = __ballot_sync(~0u, visible);
        const uint32_t mb = __ballot_sync(~0u, mar);
        const uint32_t lb0 = __ballot_sync(~0u, (lod & 1u) != 0u);
        const uint32_t lb1 = __ballot_sync(~0u, (lod & 2u) != 0u);
        if (lane == 0) {
            ballot[j][warp] = vb;
            if (i0 < n) {
                const uint64_t w = base + (uint64_t)(j * kLeafWarps + warp);
                planes[w] = vb;
                planes[stride + w] = lb0;
                planes[2 * stride + w] = lb1;
                if (marginal) marginal[i0 >> 5] = mb;
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = leaf_tile_word(ballot, s_last_start, b);
        if (lane == 0) planes[3 * stride + item] = w;
    }
}

// Launch 2: one CTA per view turns its items' tile words into carries.
constexpr int kBatchedScanThreads = 256;
__global__ void __launch_bounds__(kBatchedScanThreads) batched_tile_scan_kernel(const ViewJob* __restrict__ jobs,
                                                                               uint32_t* __restrict__ words)
{
    grid_dependents_launch();
    const ViewJob* J = jobs + blockIdx.x;
    const uint32_t lo = J->first_item;
    scan_tile_words<kBatchedScanThreads, 4>(words, lo, lo + J->num_tiles);
}

// Launch 3: one CTA per item writes its commands and counts, as the plain
// pass's write kernel does; a programmatic dependent of the scan, it reads
// only the carry after griddepcontrol.wait (the planes come from launch 1,
// complete before the scan started).
__global__ void __launch_bounds__(kLeafThreads, kWriteCtasPerSm) batched_write_kernel(const ViewJob* __restrict__ jobs,
                                                                                     uint32_t num_jobs,
                                                                                     const uint32_t* __restrict__ planes,
                                                                                     uint64_t stride, uint32_t* error)
{
    __shared__ LeafTile::Smem sm;
    extern __shared__ uint32_t s_off[];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t item = blockIdx.x;
    const ViewJob* J = jobs + warp_find_job(jobs, num_jobs, item);
    const uint32_t n = J->n, S = J->num_state_sets;
    const uint32_t tile = item - J->first_item;
    const uint32_t b = tile * (uint32_t)kLeafTile;
    if (t == 0) (void)CADR_CHECKED(item >= J->first_item && tile < max(1u, J->num_tiles), error);
    const uint32_t* off = stage_offsets(s_off, kWriteOffsetCap, J->offsets, S);
    if (t == 0 && n) cp_async_8(&sm.info[4], J->tile_region + tile);
    const uint32_t* geometry = J->geometry;
    const uint64_t base = (uint64_t)item * 64;
    uint32_t vw[kLeafIpt], l0[kLeafIpt], l1[kLeafIpt], geo[kLeafIpt];
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
        const uint32_t i = i0 + (uint32_t)lane;
        const uint64_t w = base + (uint64_t)(j * kLeafWarps + warp);
        vw[j] = i0 < n ? __ldg(planes + w) : 0u;
        l0[j] = i0 < n ? __ldg(planes + stride + w) : 0u;
        l1[j] = i0 < n ? __ldg(planes + 2 * stride + w) : 0u;
        geo[j] = i < n ? __ldg(geometry + i) : 0u;
    }
    uint32_t vis_bits = 0, lod_bits = 0;
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        vis_bits |= ((vw[j] >> lane) & 1u) << j;
        lod_bits |= (((l0[j] >> lane) & 1u) | (((l1[j] >> lane) & 1u) << 1)) << (2 * j);
        if (lane == 0) sm.ballot[j][warp] = vw[j];
    }
    uint4 ent[kLeafIpt];
    LeafTile::gather(vis_bits, lod_bits, geo, J->lods, J->num_geometries, J->num_lods, error, ent);
    grid_dependency_wait();
    if (t == 0) {
        sm.info[2] = load_relaxed_u32(planes + 3 * stride + item);
        cp_async_wait_all();
    }
    __syncthreads();
    if (n)
        LeafTile::scan_known_regions(sm);
    else
        LeafTile::scan(sm, off, S, b, n);
    LeafTile::write_ent(sm, vis_bits, ent, b, n, tile == 0, off, S, J->cmds, J->counts, error);
}

using KernelFn = void (*)(const ViewJob*, uint32_t, uint32_t, const Scratch, uint32_t*, uint64_t, uint32_t);

template <int TH>
KernelFn pick_ipt(uint32_t ipt)
{
    switch (ipt) {
    case 4: return batched_kernel<TH, 4>;
    case 8: return batched_kernel<TH, 8>;
    case 16: return batched_kernel<TH, 16>;
    }
    return nullptr;
}

KernelFn pick_kernel(uint32_t threads, uint32_t ipt)
{
    switch (threads) {
    case 128: return pick_ipt<128>(ipt);
    case 256: return pick_ipt<256>(ipt);
    case 512: return pick_ipt<512>(ipt);
    }
    return nullptr;
}

}  // namespace

uint32_t batched_tile(const cadr_tuning& tu)
{
    return tu.form == kBatchedThreeLaunch ? (uint32_t)kLeafTile : tu.block_threads * tu.items_per_thread;
}

uint64_t batched_plane_words(const cadr_tuning& tu, uint64_t total_items)
{
    return tu.form == kBatchedThreeLaunch ? 3 * batched_plane_stride(total_items) + ((total_items + 3) & ~uint64_t(3))
                                          : 0;
}

cudaError_t launch_batched_cull(const ViewJob* d_jobs, uint32_t num_jobs, uint32_t total_items, Scratch& s,
                                uint32_t* error, uint64_t spin_limit_ns, uint32_t fault, const cadr_tuning& tu,
                                uint32_t grid, cudaStream_t stream)
{
    if (tu.form == kBatchedThreeLaunch) {
        if (total_items == 0) return cudaSuccess;
        const uint64_t stride = batched_plane_stride(total_items);
        batched_classify_kernel<<<total_items, kLeafThreads, 0, stream>>>(d_jobs, num_jobs, s.planes, stride);
        batched_tile_scan_kernel<<<num_jobs, kBatchedScanThreads, 0, stream>>>(d_jobs, s.planes + 3 * stride);
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr.val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(total_items);
        cfg.blockDim = dim3(kLeafThreads);
        cfg.dynamicSmemBytes = kWriteOffsetCap * sizeof(uint32_t);
        cfg.stream = stream;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, batched_write_kernel, d_jobs, num_jobs,
                                                 (const uint32_t*)s.planes, stride, error);
        return e == cudaSuccess ? cudaGetLastError() : e;
    }
    KernelFn k = pick_kernel(tu.block_threads, tu.items_per_thread);
    if (!k) return cudaErrorInvalidValue;
    k<<<grid, tu.block_threads, kBatchedOffsetCap * sizeof(uint32_t), stream>>>(d_jobs, num_jobs, total_items, s,
                                                                             error, spin_limit_ns, fault);
    return cudaGetLastError();
}

void destroy_batched_state(cadr_context* ctx)
{
    BatchedState* b = ctx->batched;
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_jobs) cudaFree(b->d_jobs);
    if (b->h_jobs) cudaFreeHost(b->h_jobs);
    if (b->jobs_free) cudaEventDestroy(b->jobs_free);
    scratch_release(b->scratch);
    delete b;
    ctx->batched = nullptr;
}

bool tuning_valid(const cadr_tuning& t)
{
    if (t.ctas_per_sm < 1 || t.ctas_per_sm > 16) return false;
    if (t.form == kBatchedThreeLaunch) return t.block_threads == (uint32_t)kLeafThreads && t.items_per_thread == (uint32_t)kLeafIpt;
    return t.form == kBatchedPersistent && pick_kernel(t.block_threads, t.items_per_thread) != nullptr;
}

// Fills `jobs` for a batch and returns the total number of work items.
cadr_status build_jobs(const cadr_batch_view* views, uint32_t n, uint32_t tile, ViewJob* jobs, uint64_t* total)
{
    uint64_t items = 0;
    for (uint32_t v = 0; v < n; v++) {
        const cadr_batch_view& bv = views[v];
        cadr_scene* sc = bv.scene;
        if (!sc) return fail(CADR_ERR_INVALID_ARG, "cull_batched: view %u has no scene", v);
        if (!sc->committed) return fail(CADR_ERR_INVALID_ARG, "cull_batched: scene of view %u is not committed", v);
        if (!bv.counts || (!bv.cmds && sc->desc.num_drawables))
            return fail(CADR_ERR_INVALID_ARG, "cull_batched: view %u has no output buffers", v);
        ViewJob& j = jobs[v];
        std::memset(&j, 0, sizeof(j));
        j.world_sphere = reinterpret_cast<const float4*>(sc->buf.world_sphere);
        j.geometry = sc->buf.geometry;
        j.offsets = sc->buf.state_set_offsets;
        j.lods = reinterpret_cast<const uint4*>(sc->buf.lods);
        j.cmds = reinterpret_cast<uint32_t*>(bv.cmds);
        j.counts = bv.counts;
        j.marginal = bv.marginal;
        j.tile_start = sc->tile_start;
        j.tile_region = reinterpret_cast<const uint2*>(sc->tile_region);
        j.n = (uint32_t)sc->desc.num_drawables;
        j.num_state_sets = sc->desc.num_state_sets;
        j.num_geometries = sc->desc.num_geometries;
        j.num_lods = sc->desc.num_lods;
        // An empty scene still takes one item, which writes its zero counts.
        j.num_tiles = std::max<uint32_t>(1u, (uint32_t)((sc->desc.num_drawables + tile - 1) / tile));
        j.first_item = (uint32_t)items;
        j.view = to_view_const(bv.view);
        items += j.num_tiles;
        if (items >= 0xFFFF0000ull) return fail(CADR_ERR_INVALID_ARG, "cull_batched: too many work items");
    }
    *total = items;
    return CADR_OK;
}

}  // namespace cadr

using namespace cadr;

extern "C" {

CADR_API cadr_status cadr_get_tuning(cadr_context* ctx, cadr_tuning* out)
{
    if (!ctx || !out) return fail(CADR_ERR_INVALID_ARG, "get_tuning: null argument");
    *out = ctx->tuning;
    return CADR_OK;
}

CADR_API cadr_status cadr_set_tuning(cadr_context* ctx, const cadr_tuning* t)
{
    if (!ctx || !t) return fail(CADR_ERR_INVALID_ARG, "set_tuning: null argument");
    if (!tuning_valid(*t))
        return fail(CADR_ERR_INVALID_ARG, "set_tuning: unsupported block %u / items %u / ctas %u / form %u",
                    t->block_threads, t->items_per_thread, t->ctas_per_sm, t->form);
    ctx->tuning = *t;
    return CADR_OK;
}

CADR_API cadr_status cadr_cull_batched(cadr_context* ctx, const cadr_batch_view* views, uint32_t num_views,
                                       const cadr_tuning* tuning, int use_graph, cadr_stream stream)
{
    if (!ctx || (!views && num_views)) return fail(CADR_ERR_INVALID_ARG, "cull_batched: null argument");
    DeviceGuard dg(ctx->device);
    if (num_views == 0) return CADR_OK;
    const cadr_tuning tu = tuning ? *tuning : ctx->tuning;
    if (!tuning_valid(tu)) return fail(CADR_ERR_INVALID_ARG, "cull_batched: unsupported tuning");
    cudaStream_t s = pick_stream(ctx, stream);
    if (!ctx->batched) ctx->batched = new BatchedState();
    BatchedState& B = *ctx->batched;
    cudaError_t e;
    if (!B.jobs_free) {
        e = cudaEventCreateWithFlags(&B.jobs_free, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: event");
    }
    if (B.jobs_pending) {
        e = cudaEventSynchronize(B.jobs_free);  // the previous copy has read h_jobs
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: wait for job buffer");
        B.jobs_pending = false;
    }
    if (num_views > B.cap) {
        if (B.exec) cudaGraphExecDestroy(B.exec);
        if (B.graph) cudaGraphDestroy(B.graph);
        B.exec = nullptr;
        B.graph = nullptr;
        cudaDeviceSynchronize();
        if (B.d_jobs) cudaFree(B.d_jobs);
        if (B.h_jobs) cudaFreeHost(B.h_jobs);
        B.d_jobs = nullptr;
        B.h_jobs = nullptr;
        const uint32_t cap = std::max<uint32_t>(num_views, 64u);
        e = cudaMalloc(&B.d_jobs, cap * sizeof(ViewJob));
        if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&B.h_jobs), cap * sizeof(ViewJob), cudaHostAllocDefault);
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: job buffers");
        B.cap = cap;
    }
    // Scenes may have pending uploads; order them before the batch.
    for (uint32_t v = 0; v < num_views; v++) {
        cadr_status st = scene_prepare(views[v].scene, s);
        if (st != CADR_OK) return st;
    }
    uint64_t total = 0;
    cadr_status st = build_jobs(views, num_views, batched_tile(tu), B.h_jobs, &total);
    if (st != CADR_OK) return st;
    st = scratch_reserve(ctx, B.scratch, total);
    if (st == CADR_OK) st = scratch_reserve_planes(ctx, B.scratch, batched_plane_words(tu, total));
    if (st != CADR_OK) return st;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(total, (uint64_t)tu.ctas_per_sm * ctx->num_sms);
    const size_t job_bytes = num_views * sizeof(ViewJob);

    if (use_graph) {
        const bool same = B.exec && B.key_views == num_views && B.key_items == total && B.key_grid == grid &&
                          B.key_stream == s && B.key_limit == ctx->spin_limit_ns && B.key_fault == ctx->fault &&
                          std::memcmp(&B.key_tuning, &tu, sizeof(tu)) == 0;
        if (!same) {
            if (B.exec) cudaGraphExecDestroy(B.exec);
            if (B.graph) cudaGraphDestroy(B.graph);
            B.exec = nullptr;
            B.graph = nullptr;
            e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(e, "cull_batched: begin capture");
            cudaError_t e1 = cudaMemcpyAsync(B.d_jobs, B.h_jobs, job_bytes, cudaMemcpyHostToDevice, s);
            cudaError_t e2 = launch_batched_cull(B.d_jobs, num_views, (uint32_t)total, B.scratch, ctx->d_error,
                                                 ctx->spin_limit_ns, ctx->fault, tu, grid, s);
            e = cudaStreamEndCapture(s, &B.graph);
            if (e1 != cudaSuccess || e2 != cudaSuccess || e != cudaSuccess) {
                if (B.graph) cudaGraphDestroy(B.graph);
                B.graph = nullptr;
                return cuda_fail(e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e), "cull_batched: capture");
            }
            e = cudaGraphInstantiate(&B.exec, B.graph, 0);
            if (e != cudaSuccess) return cuda_fail(e, "cull_batched: instantiate");
            B.key_views = num_views;
            B.key_items = (uint32_t)total;
            B.key_grid = grid;
            B.key_tuning = tu;
            B.key_stream = s;
            B.key_limit = ctx->spin_limit_ns;
            B.key_fault = ctx->fault;
        }
        e = cudaGraphLaunch(B.exec, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: graph launch");
    } else {
        e = cudaMemcpyAsync(B.d_jobs, B.h_jobs, job_bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: job copy");
        e = launch_batched_cull(B.d_jobs, num_views, (uint32_t)total, B.scratch, ctx->d_error, ctx->spin_limit_ns,
                                ctx->fault, tu, grid, s);
        if (e != cudaSuccess) return cuda_fail(e, "cull_batched: launch");
    }
    ctx->launches += tu.form == kBatchedThreeLaunch ? 3 : 1;
    B.scratch.launches++;
    for (uint32_t v = 0; v < num_views; v++) {
        cadr_status st = scene_mark_read(views[v].scene, s);
        if (st != CADR_OK) return st;
    }
    e = cudaEventRecord(B.jobs_free, s);
    if (e != cudaSuccess) return cuda_fail(e, "cull_batched: record");
    B.jobs_pending = true;
    return CADR_OK;
}

// Autotuner: times every supported (block, items per thread, CTAs per SM)
// combination on the given batch with CUDA events (median of `reps` runs
// after one warm-up) and keeps the fastest in the context.  With a tuning
// cache set on the context, a batch whose key (batch shape, GPU, driver) is
// in the cache takes the stored pick without timing anything.
namespace {

struct TimeBatch {
    cadr_context* ctx;
    const cadr_batch_view* views;
    uint32_t num_views;
    uint32_t reps;
    cudaEvent_t a, b;
};

cadr_status time_batch(const cadr_tuning* tu, void* user, float* out_ms)
{
    TimeBatch& T = *static_cast<TimeBatch*>(user);
    cudaStream_t s = T.ctx->stream;
    std::vector<float> ts;
    for (uint32_t r = 0; r <= T.reps; r++) {
        cudaEventRecord(T.a, s);
        const cadr_status st = cadr_cull_batched(T.ctx, T.views, T.num_views, tu, 0, s);
        cudaEventRecord(T.b, s);
        if (st != CADR_OK) return st;
        const cudaError_t e = cudaEventSynchronize(T.b);
        if (e != cudaSuccess) return cuda_fail(e, "autotune: wait");
        float ms = 0;
        cudaEventElapsedTime(&ms, T.a, T.b);
        if (r) ts.push_back(ms);
    }
    std::sort(ts.begin(), ts.end());
    *out_ms = ts[ts.size() / 2];
    return CADR_OK;
}

// The cache key of a batch: the GPU (name, SMs, compute capability), the
// driver, this library's ABI, and the batch's shape (per view: the scene's
// drawables, StateSets and LODs), the shape hashed with FNV-1a.
std::string tuning_key(const cadr_context* ctx, const cadr_batch_view* views, uint32_t n)
{
    cudaDeviceProp p{};
    cudaGetDeviceProperties(&p, ctx->device);
    int driver = 0;
    cudaDriverGetVersion(&driver);
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int k = 0; k < 8; k++) {
            h ^= (v >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    };
    uint64_t drawables = 0;
    for (uint32_t v = 0; v < n; v++) {
        const cadr_scene_desc& d = views[v].scene->desc;
        mix(d.num_drawables);
        mix(d.num_state_sets);
        mix(d.num_lods);
        drawables += d.num_drawables;
    }
    std::string name;
    for (const char* c = p.name; *c; c++) name += (*c == '"' || *c == '\\') ? '_' : *c;
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s|sms=%d|cc=%d.%d|driver=%d|abi=%d|views=%u|drawables=%llu|shape=%016llx",
                  name.c_str(), p.multiProcessorCount, p.major, p.minor, driver, cadr_abi_version(), n,
                  (unsigned long long)drawables, (unsigned long long)h);
    return buf;
}

}  // namespace

CADR_API cadr_status cadr_context_set_tuning_cache(cadr_context* ctx, const char* path)
{
    if (!ctx) return fail(CADR_ERR_INVALID_ARG, "set_tuning_cache: null context");
    ctx->tuning_cache = path ? path : "";
    return CADR_OK;
}

CADR_API cadr_status cadr_autotune_batched(cadr_context* ctx, const cadr_batch_view* views, uint32_t num_views,
                                           uint32_t reps, cadr_tuning* best, float* best_ms)
{
    if (!ctx || !views || num_views == 0 || !best) return fail(CADR_ERR_INVALID_ARG, "autotune: bad argument");
    DeviceGuard dg(ctx->device);
    for (uint32_t v = 0; v < num_views; v++)
        if (!views[v].scene) return fail(CADR_ERR_INVALID_ARG, "autotune: view %u has no scene", v);
    TimeBatch T{ctx, views, num_views, reps ? reps : 5u, nullptr, nullptr};
    cudaError_t e = cudaEventCreate(&T.a);
    if (e == cudaSuccess) e = cudaEventCreate(&T.b);
    if (e != cudaSuccess) return cuda_fail(e, "autotune: events");
    const std::string key = tuning_key(ctx, views, num_views);
    cadr_tuning pick = ctx->tuning;
    float ms = 0;
    const cadr_status st = cadr_autotune_with(ctx->tuning_cache.empty() ? nullptr : ctx->tuning_cache.c_str(),
                                              key.c_str(), time_batch, &T, &pick, &ms, nullptr);
    cudaEventDestroy(T.a);
    cudaEventDestroy(T.b);
    if (st != CADR_OK) return st;
    if (!tuning_valid(pick)) return fail(CADR_ERR_INVALID_ARG, "autotune: cached tuning is not supported");
    ctx->tuning = pick;
    *best = pick;
    if (best_ms) *best_ms = ms;
    return CADR_OK;
}

}  // extern "C"
