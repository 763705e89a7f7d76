// cull.cu - Tier B kernels: hierarchy propagation, the fused leaf pass
// (world matrix, bounding sphere, frustum cull, LOD, per-StateSet
// compaction) and the batched sphere cull.
//
// Compaction is a single-pass segmented scan with decoupled lookback over
// dynamically numbered tiles (a tile's predecessors were started before it,
// so they are resident and its wait always ends); each wait is bounded by a
// time limit after which the tile records CADR_DEVERR_LOOKBACK_TIMEOUT and
// continues, so no pass can hang the device.  Output order inside a
// StateSet region is ascending drawable order: deterministic, no atomics on
// the output.
#include <algorithm>
#include <atomic>

#include "compact.cuh"
#include "kernels.cuh"

namespace cadr {

namespace {

__device__ __forceinline__ void load_mat(const float4* __restrict__ p, float4& c0, float4& c1,
                                         float4& c2, float4& c3)
{
    c0 = ld_nc_f4(p + 0);
    c1 = ld_nc_f4(p + 1);
    c2 = ld_nc_f4(p + 2);
    c3 = ld_nc_f4(p + 3);
}

using LeafTile = Tile<kLeafThreads, kLeafIpt>;

#ifndef CADR_LEAF_CTAS_PER_SM
#define CADR_LEAF_CTAS_PER_SM 4
#endif
constexpr int kLeafCtasPerSm = CADR_LEAF_CTAS_PER_SM;
// Rows whose LOD entries one thread holds at a time in the compaction.
constexpr int kLeafChunk = kLeafIpt < 8 ? kLeafIpt : 8;
static_assert(kLeafIpt == kLeafChunk || kLeafIpt == 2 * kLeafChunk, "one or two compaction chunks");

// Shared-memory record of a streamed tile that the compaction reads:
// per item its geometry id and LOD (ballots and scan results are in the
// tile's LeafTile::Smem).
struct LeafStash {
    uint32_t geo[kLeafTile];
    uint8_t lod[kLeafTile];
};

// World matrix records leave through a 2 KB staging block per warp, so
// that each store instruction of a warp writes 512 contiguous bytes:
// stored with per-lane 64-byte strides, the records reach only about 90%
// of the HBM bandwidth of contiguous stores (strided loads lose nothing).
// Chunk q of a row's 128 float4 (column q & 3 of record q >> 2) sits at
// position q ^ ((q >> 3) & 3), so that both the record-order writes
// (chunks 4 lane + c) and the chunk-order reads (lane + 32k) of each
// quarter-warp cover all 32 banks once.
__device__ __forceinline__ uint32_t xpose_pos(uint32_t q) { return q ^ ((q >> 3) & 3u); }

// Streams the drawables [b, b + kLeafTile): world matrix, world sphere
// and, with kCull, the classification.  Item j of thread t is drawable
// b + j*kLeafThreads + t, i.e. lane t%32 of row j of warp t/32; xb is the
// warp's staging block.  With kCull, visibility ballots go to sm, geometry
// ids and LODs to st at position j*kLeafThreads + t.
template <bool kCull>
__device__ __forceinline__ void stream_tile(const LeafArgs& a, uint32_t b, LeafTile::Smem* sm, LeafStash* st,
                                            float4* xb)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
        const uint32_t i = i0 + (uint32_t)lane;
        bool visible = false, marginal = false;
        uint32_t lod = 0, geo = 0;
        if (i0 < a.n) {
            // The previous row's reads of xb are done before it is rewritten.
            __syncwarp();
            if (i < a.n) {
                float4 l0, l1, l2, l3, w0, w1, w2, w3;
                load_mat(a.local + (size_t)i * 4, l0, l1, l2, l3);
                const float4 sp = ld_nc_f4(a.sphere + i);
                if (kCull) geo = ld_nc_u32(a.geometry + i);
                if (a.parent) {
                    uint32_t p = ld_nc_u32(a.parent + i);
                    if (p >= a.num_parents) {
                        atomicOr(a.error, CADR_DEVERR_BAD_INDEX);
                        p = 0;
                    }
                    const float4* pp = a.parent_world + (size_t)p * 4;
                    const float4 p0 = __ldg(pp), p1 = __ldg(pp + 1), p2 = __ldg(pp + 2), p3 = __ldg(pp + 3);
                    w0 = mat_col(p0, p1, p2, p3, l0);
                    w1 = mat_col(p0, p1, p2, p3, l1);
                    w2 = mat_col(p0, p1, p2, p3, l2);
                    w3 = mat_col(p0, p1, p2, p3, l3);
                } else {
                    w0 = l0;
                    w1 = l1;
                    w2 = l2;
                    w3 = l3;
                }
                xb[xpose_pos(4u * lane + 0)] = w0;
                xb[xpose_pos(4u * lane + 1)] = w1;
                xb[xpose_pos(4u * lane + 2)] = w2;
                xb[xpose_pos(4u * lane + 3)] = w3;
                const float4 ws = transform_sphere(w0, w1, w2, w3, sp);
                if (a.world_sphere) st_cs_f4(a.world_sphere + i, ws);
                if (kCull) classify(a.view, ws, a.num_lods, visible, marginal, lod);
            }
            __syncwarp();
            const uint32_t cnt = min((uint32_t)kWarp, a.n - i0);
            float4* wp = a.world + (size_t)i0 * 4;
#pragma unroll
            for (uint32_t k = 0; k < 4; k++) {
                const uint32_t q = (uint32_t)lane + 32u * k;
                if ((q >> 2) < cnt) st_cs_f4(wp + q, xb[xpose_pos(q)]);
            }
        }
        if (kCull) {
            const uint32_t vb = __ballot_sync(~0u, visible);
            const uint32_t mb = __ballot_sync(~0u, marginal);
            if (lane == 0) {
                sm->ballot[j][warp] = vb;
                if (a.marginal && i0 < a.n) a.marginal[i0 >> 5] = mb;
            }
            st->geo[j * kLeafThreads + t] = geo;
            st->lod[j * kLeafThreads + t] = (uint8_t)lod;
        }
    }
}

// Leaf level without culling: one CTA per tile.
__global__ void __launch_bounds__(kLeafThreads, 4) leaf_propagate_kernel(const LeafArgs a)
{
    __shared__ float4 xb[kLeafThreads / kWarp][4 * kWarp];
    stream_tile<false>(a, blockIdx.x * (uint32_t)kLeafTile, nullptr, nullptr, xb[threadIdx.x >> 5]);
}

// Visibility bits of the thread's items in a streamed tile (bit j: row j).
__device__ __forceinline__ uint32_t tile_vis_bits(const LeafTile::Smem& sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v = 0;
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) v |= ((sm.ballot[j][warp] >> lane) & 1u) << j;
    return v;
}

// LOD-table entries of the thread's visible items in rows [J0, J0 + kLeafChunk).
template <int J0>
__device__ __forceinline__ void gather_rows(const LeafArgs& a, const LeafStash& st, uint32_t vis_bits,
                                            uint4 (&ent)[kLeafChunk])
{
    const int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < kLeafChunk; j++) {
        ent[j] = make_uint4(0u, 0u, 0u, 0u);
        if (!((vis_bits >> (J0 + j)) & 1u)) continue;
        uint32_t g = st.geo[(J0 + j) * kLeafThreads + t];
        if (g >= a.num_geometries) {
            atomicOr(a.error, CADR_DEVERR_BAD_INDEX);
            g = 0;
        }
        ent[j] = __ldg(a.lods + (size_t)g * a.num_lods + st.lod[(J0 + j) * kLeafThreads + t]);
    }
}

// The fused plain pass, persistent: every CTA takes tiles from the pass's
// tile counter (so in ascending order across the grid) until none is left.
// A tile's aggregate is published as soon as its drawables are streamed;
// its lookback and command writes are deferred until the CTA has streamed
// its next tile.  By then the tiles before it have published long ago, so
// the lookback walks published states instead of waiting for neighbours
// that are still streaming, and the deferred tile's LOD gathers overlap
// that walk.  Deferral cannot deadlock: a tile's aggregate waits only for
// the lookback of a lower tile of the same CTA, which waits only for the
// aggregates of tiles lower still, and tile 0 publishes its prefix at once.
// Shared memory: two tile records (current, deferred), the warps' staging
// blocks, then the staged StateSet offsets.
__global__ void __launch_bounds__(kLeafThreads, kLeafCtasPerSm) leaf_cull_kernel(const LeafArgs a, const Scratch s)
{
    __shared__ LeafTile::Smem sm[2];
    __shared__ uint32_t s_tile;
    extern __shared__ __align__(16) uint32_t s_dyn[];
    LeafStash* stash = reinterpret_cast<LeafStash*>(s_dyn);
    float4* xbs = reinterpret_cast<float4*>(stash + 2);
    const int t = threadIdx.x, warp = t >> 5;
    const uint32_t tiles = (a.n + (uint32_t)kLeafTile - 1) / (uint32_t)kLeafTile;
    constexpr uint32_t kNone = 0xffffffffu;

    if (t == 0) {
        s_tile = atomicAdd(&s.ctl->tile_counter, 1u);
        const uint32_t epoch = load_relaxed_u32(&s.ctl->epoch);
        sm[0].info[1] = epoch;
        sm[1].info[1] = epoch;
    }
    const uint32_t* off = stage_offsets(reinterpret_cast<uint32_t*>(xbs + kLeafThreads * 4), a.off_cap, a.offsets,
                                        a.num_state_sets);
    __syncthreads();
    uint32_t tile = s_tile, pend = kNone;
    int p = 0;
    for (;;) {
        const bool cur = tile < tiles;
        const uint32_t b = tile * (uint32_t)kLeafTile;
        if (cur) {
            stream_tile<true>(a, b, &sm[p], &stash[p], xbs + warp * 4 * kWarp);
            __syncthreads();
            LeafTile::scan(sm[p], off, a.num_state_sets, b, a.n);
        }
        if (pend == kNone && !cur) break;
        // Deferred tile: LOD gathers by every thread, lookback by warp 0
        // after it has published the current tile's aggregate.
        uint32_t vis_bits = 0;
        uint4 ent[kLeafChunk];
        if (pend != kNone) {
            vis_bits = tile_vis_bits(sm[p ^ 1]);
            gather_rows<0>(a, stash[p ^ 1], vis_bits, ent);
        }
        if (warp == 0) {
            if (cur && t == 0) LeafTile::publish(sm[p], s.tile_state, tile, 0, off, b, a.fault);
            if (pend != kNone) LeafTile::resolve(sm[p ^ 1], s.tile_state, pend, 0, a.spin_limit_ns, a.error);
        }
        __syncthreads();
        if (pend != kNone) {
            const uint32_t pb = pend * (uint32_t)kLeafTile;
            LeafTile::write_cmds<0, kLeafChunk>(sm[p ^ 1], vis_bits, ent, pb, off, a.cmds);
            if constexpr (kLeafIpt > kLeafChunk) {
                // The second chunk: rows [kLeafIpt - kLeafChunk, kLeafIpt).
                constexpr int J0 = kLeafIpt - kLeafChunk;
                gather_rows<J0>(a, stash[p ^ 1], vis_bits, ent);
                LeafTile::write_cmds<J0, kLeafIpt>(sm[p ^ 1], vis_bits, ent, pb, off, a.cmds);
            }
            LeafTile::write_counts(sm[p ^ 1], pb, a.n, pend == 0, off, a.num_state_sets, a.counts);
        }
        if (!cur) break;
        // The current tile becomes the deferred one.
        if (t == 0) s_tile = atomicAdd(&s.ctl->tile_counter, 1u);
        __syncthreads();
        pend = tile;
        tile = s_tile;
        p ^= 1;
    }
    if (t == 0) finish_pass(s.ctl);
}

// Internal level propagation.  With `staged`, the CTA's run of parents
// [parent[first], parent[last]] is brought into shared memory by one bulk
// (TMA) copy completed on an mbarrier; otherwise parents are gathered.
constexpr uint32_t kMaxStaged = 256;

__global__ void __launch_bounds__(kPropThreads) propagate_kernel(
    const float4* __restrict__ pw, uint32_t np, const float4* __restrict__ local,
    const uint32_t* __restrict__ parent, uint32_t n, float4* __restrict__ world, int staged,
    uint32_t* error, uint64_t limit_ns)
{
    __shared__ __align__(128) float4 s_par[kMaxStaged * 4];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_plo, s_cnt;
    __shared__ int s_ok;

    const uint32_t b = blockIdx.x * (uint32_t)kPropThreads;
    const uint32_t i = b + threadIdx.x;
    bool use_stage = false;
    if (staged) {
        if (threadIdx.x == 0) {
            const uint32_t last = min(b + (uint32_t)kPropThreads, n) - 1;
            const uint32_t plo = __ldg(parent + b), phi = __ldg(parent + last);
            const uint32_t cnt = phi - plo + 1;
            const int ok = (phi >= plo) && (phi < np) && (cnt <= kMaxStaged);
            s_plo = plo;
            s_cnt = cnt;
            s_ok = ok;
            if (ok) {
                mbar_init(&s_bar, 1);
                mbar_arrive_expect_tx(&s_bar, cnt * 64u);
                bulk_copy_g2s(s_par, pw + (size_t)plo * 4, cnt * 64u, &s_bar);
            }
        }
        __syncthreads();
        use_stage = s_ok != 0;
        if (use_stage && !mbar_wait_bounded(&s_bar, 0, limit_ns)) {
            if (threadIdx.x == 0) atomicOr(error, CADR_DEVERR_MBARRIER_TIMEOUT);
            mbar_wait_bounded(&s_bar, 0, limit_ns);  // let an in-flight copy land before exit
            return;
        }
    }
    if (i >= n) return;
    uint32_t p = __ldg(parent + i);
    if (p >= np) {
        atomicOr(error, CADR_DEVERR_BAD_INDEX);
        p = 0;
    }
    float4 p0, p1, p2, p3;
    const uint32_t rel = p - s_plo;
    if (use_stage && rel < s_cnt) {
        p0 = s_par[rel * 4 + 0];
        p1 = s_par[rel * 4 + 1];
        p2 = s_par[rel * 4 + 2];
        p3 = s_par[rel * 4 + 3];
    } else {
        const float4* pp = pw + (size_t)p * 4;
        p0 = __ldg(pp);
        p1 = __ldg(pp + 1);
        p2 = __ldg(pp + 2);
        p3 = __ldg(pp + 3);
    }
    float4 l0, l1, l2, l3;
    load_mat(local + (size_t)i * 4, l0, l1, l2, l3);
    float4* wp = world + (size_t)i * 4;
    wp[0] = mat_col(p0, p1, p2, p3, l0);
    wp[1] = mat_col(p0, p1, p2, p3, l1);
    wp[2] = mat_col(p0, p1, p2, p3, l2);
    wp[3] = mat_col(p0, p1, p2, p3, l3);
}

}  // namespace

cudaError_t launch_propagate(const float4* parent_world, uint32_t num_parents, const float4* local,
                             const uint32_t* parent, uint32_t n, float4* world, int staged,
                             uint32_t* error, uint64_t spin_limit_ns, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    const uint32_t grid = (n + kPropThreads - 1) / kPropThreads;
    propagate_kernel<<<grid, kPropThreads, 0, stream>>>(parent_world, num_parents, local, parent, n,
                                                        world, staged, error, spin_limit_ns);
    return cudaGetLastError();
}

cudaError_t launch_leaf_propagate(const LeafArgs& a, cudaStream_t stream)
{
    if (a.n == 0) return cudaSuccess;
    const uint32_t grid = (a.n + kLeafTile - 1) / kLeafTile;
    leaf_propagate_kernel<<<grid, kLeafThreads, 0, stream>>>(a);
    return cudaGetLastError();
}

// StateSet offsets are staged in shared memory up to this many entries.
constexpr uint32_t kLeafOffsetCap = 4096;
constexpr size_t kLeafFixedSmem = 2 * sizeof(LeafStash) + kLeafThreads * 4 * sizeof(float4);
constexpr size_t kLeafMaxSmem = kLeafFixedSmem + kLeafOffsetCap * sizeof(uint32_t);
constexpr int kMaxDevices = 64;
std::atomic<bool> g_leaf_attr_set[kMaxDevices];

cudaError_t launch_leaf_cull(const LeafArgs& a, Scratch& s, cudaStream_t stream)
{
    if (a.n == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_leaf_attr_set[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(leaf_cull_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLeafMaxSmem);
        if (e != cudaSuccess) return e;
        g_leaf_attr_set[dev].store(true, std::memory_order_release);
    }
    LeafArgs b = a;
    b.off_cap = kLeafOffsetCap;
    const size_t smem = kLeafFixedSmem +
                        ((a.num_state_sets + 1 <= kLeafOffsetCap) ? a.num_state_sets + 1 : 0) * sizeof(uint32_t);
    // Persistent grid: the CTAs resident at once (at most kLeafCtasPerSm per
    // SM by the launch bounds).  Any grid size is correct, since running
    // CTAs take the tiles in order.
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, leaf_cull_kernel, kLeafThreads, smem);
    if (e != cudaSuccess) return e;
    const uint32_t tiles = (a.n + kLeafTile - 1) / kLeafTile;
    const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sms * (uint32_t)std::max(per_sm, 1));
    leaf_cull_kernel<<<grid, kLeafThreads, smem, stream>>>(b, s);
    return cudaGetLastError();
}

}  // namespace cadr
