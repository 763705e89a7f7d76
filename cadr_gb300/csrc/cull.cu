// cull.cu - Tier B kernels of the plain pass: hierarchy propagation and
// the leaf pass (world matrix, bounding sphere, frustum cull, LOD,
// per-StateSet compaction).
//
// The leaf pass is a reduce-then-scan over tiles of 2,048 drawables in
// three launches: the stream kernel computes world matrices, world spheres
// and the classification, and leaves per tile one (count, region-start)
// word and per 32 drawables the visibility and LOD bits; one CTA scans the
// tile words into per-tile carries; the write kernel turns the bits and
// carries into commands and counts.  No kernel waits for another CTA, so
// the plain pass has no spin-waits at all.  Output order inside a StateSet
// region is ascending drawable order: deterministic, no atomics on the
// output.
#include <algorithm>

#include "compact.cuh"
#include "kernels.cuh"

namespace cadr {

namespace {

// A 64-byte matrix record in two 256-bit loads (records are 32-byte
// aligned: every array sits at a 256-byte offset of the scene arena).
__device__ __forceinline__ void load_mat(const float4* __restrict__ p, float4& c0, float4& c1,
                                         float4& c2, float4& c3)
{
    ld_nc_f8(p, c0, c1);
    ld_nc_f8(p + 2, c2, c3);
}


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
// warp's staging block.  With kCull, row j's visibility ballot goes to
// ballot[j][warp] and, with the LOD bits, to word 8 warp + j of the tile's
// 64 in each plane; the marginal flags go out in drawable order.
template <bool kCull>
__device__ __forceinline__ void stream_tile(const LeafArgs& a, uint32_t b, uint32_t (*ballot)[kLeafWarps],
                                            float4* xb)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t words = (uint32_t)leaf_plane_stride(a.n);
    // The parent indices of all rows are loaded first, so that each row's
    // parent-matrix gather leaves with its own loads instead of one memory
    // round trip after them.
    uint32_t par[kLeafIpt];
    if (a.parent) {
#pragma unroll
        for (int j = 0; j < kLeafIpt; j++) {
            const uint32_t i = b + (uint32_t)(j * kLeafThreads + t);
            par[j] = i < a.n ? ld_nc_u32(a.parent + i) : 0u;
        }
    }
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
        const uint32_t i = i0 + (uint32_t)lane;
        bool visible = false, marginal = false;
        uint32_t lod = 0;
        if (i0 < a.n) {
            // The previous row's reads of xb are done before it is rewritten.
            __syncwarp();
            if (i < a.n) {
                float4 l0, l1, l2, l3, w0, w1, w2, w3;
                load_mat(a.local + (size_t)i * 4, l0, l1, l2, l3);
                const float4 sp = ld_nc_f4(a.sphere + i);
                if (a.parent) {
                    // Launched as a programmatic dependent of the last
                    // level kernel, the stream kernel reads that level's
                    // world matrices only once it has completed; the loads
                    // above (parent indices, the first row's records) and
                    // the tile's region start overlap its tail.  Without
                    // the launch attribute this is a no-op.
                    if (j == 0) grid_dependency_wait();
                    uint32_t p = par[j];
                    if (p >= a.num_parents) {
                        atomicOr(a.error, CADR_DEVERR_BAD_INDEX);
                        p = 0;
                    }
                    float4 p0, p1, p2, p3;
                    load_mat(a.parent_world + (size_t)p * 4, p0, p1, p2, p3);
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
            const uint32_t lb0 = __ballot_sync(~0u, (lod & 1u) != 0u);
            const uint32_t lb1 = __ballot_sync(~0u, (lod & 2u) != 0u);
            if (lane == 0) {
                ballot[j][warp] = vb;
                if (i0 < a.n) {
                    const uint32_t w = i0 >> 5;
                    const uint32_t wt = (i0 >> 11) * 64u + (uint32_t)warp * 8u + (uint32_t)j;
                    if (CADR_CHECKED(wt < words, a.error)) {
                        a.planes[wt] = vb;
                        a.planes[words + wt] = lb0;
                        a.planes[2 * words + wt] = lb1;
                    }
                    if (a.marginal && CADR_CHECKED(w < (a.n + 31u) / 32u, a.error)) a.marginal[w] = mb;
                }
            }
        }
    }
}

// Leaf level without culling: one CTA per tile.
__global__ void __launch_bounds__(kLeafThreads, 4) leaf_propagate_kernel(const LeafArgs a)
{
    __shared__ float4 xb[kLeafWarps][4 * kWarp];
    stream_tile<false>(a, blockIdx.x * (uint32_t)kLeafTile, nullptr, xb[threadIdx.x >> 5]);
}

// Plain pass, launch 1 of 3: one CTA per tile streams its drawables
// (world matrices, world spheres, classification into the planes) and
// writes the tile word.  No CTA waits for another.
__global__ void __launch_bounds__(kLeafThreads, 4) leaf_stream_kernel(const LeafArgs a)
{
    __shared__ float4 xb[kLeafWarps][4 * kWarp];
    __shared__ uint32_t ballot[kLeafIpt][kLeafWarps];
    __shared__ uint32_t s_last_start;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t tile = blockIdx.x, b = tile * (uint32_t)kLeafTile;
    // Start of the region holding the tile's last drawable (from the
    // scene's per-tile table); the load overlaps the stream.
    if (t == 0) s_last_start = __ldg(a.tile_start + tile);
    stream_tile<true>(a, b, ballot, xb[warp]);
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = leaf_tile_word(ballot, s_last_start, b);
        if (lane == 0) a.tile_words[tile] = w;
    }
}

// Plain pass, launch 2 of 3, one CTA: replaces every tile word by the
// tile's carry (scan_tile_words).  It lets its dependent (the write kernel)
// launch at once: that kernel reads the carries only after
// griddepcontrol.wait, which returns when this grid has completed and its
// writes are visible.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;

__global__ void __launch_bounds__(kScanThreads) leaf_tile_scan_kernel(uint32_t* __restrict__ words, uint32_t tiles)
{
    grid_dependents_launch();
    scan_tile_words<kScanThreads, kScanPer, true>(words, 0u, tiles);
}


// Plain pass, launch 3 of 3: one CTA per tile writes the commands and
// counts from the planes and the tile's carry.  No CTA waits for another.
// It is launched as a programmatic dependent of the tile scan: everything
// but the carry (the planes, the geometry ids, the offsets, the LOD-table
// gathers) is loaded while the scan still runs, and only the carry is read
// after griddepcontrol.wait.  A warp's 8 row words of a plane are two
// 16-byte loads.  The loads are independent of one another,
// so a tile costs about two memory round trips.  With kShard (a shard of a
// pass split over devices) the commands are placed by a.shard and the
// counts, written by the region-count kernel before, are left alone.
template <bool kShard>
__global__ void __launch_bounds__(kLeafThreads, kWriteCtasPerSm) leaf_write_kernel(const LeafArgs a)
{
    __shared__ LeafTile::Smem sm;
    extern __shared__ uint32_t s_off[];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t tile = blockIdx.x, b = tile * (uint32_t)kLeafTile;
    const uint32_t stride = (uint32_t)leaf_plane_stride(a.n);
    const uint32_t* off = stage_offsets(s_off, a.off_cap, a.offsets, a.num_state_sets);
    // The tile's first and last regions, from the scene's per-tile table,
    // straight into info[4], info[5].
    if (t == 0) cp_async_8(&sm.info[4], a.tile_region + tile);
    uint32_t vw[kLeafIpt], l0[kLeafIpt], l1[kLeafIpt], geo[kLeafIpt];
    {
        const uint4* pv = reinterpret_cast<const uint4*>(a.planes + tile * 64u + (uint32_t)warp * 8u);
        const uint32_t q = stride / 4u;
        const uint4 v0 = __ldg(pv), v1 = __ldg(pv + 1), a0 = __ldg(pv + q), a1 = __ldg(pv + q + 1),
                    c0 = __ldg(pv + 2 * q), c1 = __ldg(pv + 2 * q + 1);
        vw[0] = v0.x; vw[1] = v0.y; vw[2] = v0.z; vw[3] = v0.w; vw[4] = v1.x; vw[5] = v1.y; vw[6] = v1.z; vw[7] = v1.w;
        l0[0] = a0.x; l0[1] = a0.y; l0[2] = a0.z; l0[3] = a0.w; l0[4] = a1.x; l0[5] = a1.y; l0[6] = a1.z; l0[7] = a1.w;
        l1[0] = c0.x; l1[1] = c0.y; l1[2] = c0.z; l1[3] = c0.w; l1[4] = c1.x; l1[5] = c1.y; l1[6] = c1.z; l1[7] = c1.w;
    }
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
        const uint32_t i = i0 + (uint32_t)lane;
        if (i0 >= a.n) vw[j] = l0[j] = l1[j] = 0u;
        geo[j] = i < a.n ? __ldg(a.geometry + i) : 0u;
    }
    uint32_t vis_bits = 0, lod_bits = 0;
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        vis_bits |= ((vw[j] >> lane) & 1u) << j;
        lod_bits |= (((l0[j] >> lane) & 1u) | (((l1[j] >> lane) & 1u) << 1)) << (2 * j);
        if (lane == 0) sm.ballot[j][warp] = vw[j];
    }
    uint4 ent[kLeafIpt];
    LeafTile::gather(vis_bits, lod_bits, geo, a.lods, a.num_geometries, a.num_lods, a.error, ent);
    grid_dependency_wait();
    if (t == 0) {
        sm.info[2] = load_relaxed_u32(a.tile_words + tile);
        cp_async_wait_all();
#ifdef CADR_BOUNDS_CHECK
        // The scene's table against the offsets: the tile's first and last
        // drawables lie in its first and last regions.  (The command writes
        // check their own regions; this only reports a stale table.)
        const uint32_t rf = sm.info[4], rl = sm.info[5], e = min(b + (uint32_t)kLeafTile, a.n) - 1u;
        (void)CADR_CHECKED(rf <= rl && rl < a.num_state_sets && in_region(a.offsets, rf, b, b) &&
                               in_region(a.offsets, rl, e, e),
                           a.error);
#endif
    }
    __syncthreads();
    LeafTile::scan_known_regions(sm);
    if (kShard)
        LeafTile::write_cmds<0, kLeafIpt, true>(sm, vis_bits, ent, b, a.n, off, a.cmds, a.error, a.shard);
    else
        LeafTile::write_ent(sm, vis_bits, ent, b, a.n, tile == 0, off, a.num_state_sets, a.cmds, a.counts, a.error);
}

// Sharded pass: the visible drawables of every StateSet region, one warp
// per region, from the visibility plane and the carries the tile scan left
// (the carry of a tile counts the visible drawables of the region holding
// the tile's first drawable that precede the tile).  A region that starts
// before the tile of its last drawable takes that tile's carry and counts
// the bits from the tile start; one that starts inside it counts its own
// bits; either way at most one tile of 2,048 bits is read.
__global__ void __launch_bounds__(256) leaf_region_count_kernel(const uint32_t* __restrict__ planes,
                                                                const uint32_t* __restrict__ carries,
                                                                const uint32_t* __restrict__ offsets, uint32_t S,
                                                                uint32_t* __restrict__ counts)
{
    const uint32_t region = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (region >= S) return;
    const uint32_t s0 = __ldg(offsets + region), e = __ldg(offsets + region + 1);
    uint32_t c = 0, base = 0;
    if (e > s0) {
        const uint32_t last_tile = (e - 1) / (uint32_t)kLeafTile;
        const uint32_t tb = last_tile * (uint32_t)kLeafTile;
        uint32_t from = s0;
        if (s0 < tb) {
            from = tb;
            base = __ldg(carries + last_tile);
        }
        for (uint32_t w = (from >> 5) + lane; w <= ((e - 1) >> 5); w += 32u) {
            // word w in drawable order (tile, row j, warp) is stored at
            // tile word 8 warp + j
            uint32_t v = __ldg(planes + ((w & ~63u) | ((w & 7u) << 3) | ((w >> 3) & 7u)));
            const uint32_t lo = w * 32u;
            if (from > lo) v &= ~0u << (from - lo);      // from - lo in 1..31
            if (e < lo + 32u) v &= (1u << (e - lo)) - 1u;  // e - lo in 1..31
            c += __popc(v);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(~0u, c, o);
    if (lane == 0) counts[region] = base + c;
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

    // A programmatic dependent (the next level, or the plain pass's stream
    // kernel after the last level) may launch now: it reads this level's
    // world matrices only after griddepcontrol.wait.
    grid_dependents_launch();
    const uint32_t b = blockIdx.x * (uint32_t)kPropThreads;
    const uint32_t i = b + threadIdx.x;
    // This node's inputs do not depend on the previous level: they are in
    // flight while it finishes (when this kernel is its programmatic
    // dependent; otherwise the wait below is a no-op).
    uint32_t p = 0;
    float4 l0 = {}, l1 = {}, l2 = {}, l3 = {};
    if (i < n) {
        p = __ldg(parent + i);
        load_mat(local + (size_t)i * 4, l0, l1, l2, l3);
    }
    uint32_t plo = 0, phi = 0;
    if (staged && threadIdx.x == 0) {
        const uint32_t last = min(b + (uint32_t)kPropThreads, n) - 1;
        plo = __ldg(parent + b);
        phi = __ldg(parent + last);
    }
    grid_dependency_wait();
    bool use_stage = false;
    if (staged) {
        if (threadIdx.x == 0) {
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
    // Default-cached stores: the next level (or the leaf pass) gathers
    // these matrices as parents while they are still in L2.
    float4* wp = world + (size_t)i * 4;
    st_f8(wp, mat_col(p0, p1, p2, p3, l0), mat_col(p0, p1, p2, p3, l1));
    st_f8(wp + 2, mat_col(p0, p1, p2, p3, l2), mat_col(p0, p1, p2, p3, l3));
}

constexpr int kFoldThreads = 256;

__host__ __device__ constexpr uint32_t pad16_words(uint32_t n) { return (n + 3u) & ~3u; }

// Shared memory of the folded levels: 64 B per node (level 0 and every
// folded level), then the parent indices of the folded levels (each level
// padded to 16 bytes).
constexpr size_t kFoldSmemWords = kFoldMaxNodes * 16 + kFoldMaxNodes + 4 * CADR_MAX_LEVELS;

__global__ void __launch_bounds__(kFoldThreads) propagate_small_levels_kernel(const FoldArgs a)
{
    __shared__ __align__(128) float4 s_mat[kFoldSmemWords / 4];  // level 0, then each folded level: 4 float4 per node
    __shared__ __align__(8) uint64_t s_bar;
    // The next level kernel (or the stream kernel) may launch now: it reads
    // these levels' world matrices only after griddepcontrol.wait.
    grid_dependents_launch();
    uint32_t total = a.n0, par_words = 0;
    for (uint32_t l = 0; l < a.count; l++) {
        total += a.lvl[l].n;
        par_words += pad16_words(a.lvl[l].n);
    }
    uint32_t* s_par = reinterpret_cast<uint32_t*>(s_mat + 4 * (size_t)total);
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        mbar_arrive_expect_tx(&s_bar, total * 64u + par_words * 4u);
        bulk_copy_g2s(s_mat, a.world0, a.n0 * 64u, &s_bar);
        uint32_t m = a.n0, po = 0;
        for (uint32_t l = 0; l < a.count; l++) {
            const uint32_t n = a.lvl[l].n;
            bulk_copy_g2s(s_mat + 4 * (size_t)m, a.lvl[l].local, n * 64u, &s_bar);
            // Padded to 16 bytes: the arena rounds every array up to 256.
            bulk_copy_g2s(s_par + po, a.lvl[l].parent, pad16_words(n) * 4u, &s_bar);
            m += n;
            po += pad16_words(n);
        }
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&s_bar, 0, a.limit_ns);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicOr(a.error, CADR_DEVERR_MBARRIER_TIMEOUT);
            mbar_wait_bounded(&s_bar, 0, a.limit_ns);  // let in-flight copies land before exit
        }
        return;
    }
    uint32_t prev = 0, np = a.n0, m = a.n0, po = 0;
    for (uint32_t l = 0; l < a.count; l++) {
        const uint32_t n = a.lvl[l].n;
        float4* world = a.lvl[l].world;
        for (uint32_t i = threadIdx.x; i < n; i += kFoldThreads) {
            uint32_t p = s_par[po + i];
            if (p >= np) {
                atomicOr(a.error, CADR_DEVERR_BAD_INDEX);
                p = 0;
            }
            const float4* P = s_mat + 4 * (size_t)(prev + p);
            float4* C = s_mat + 4 * (size_t)(m + i);
            const float4 p0 = P[0], p1 = P[1], p2 = P[2], p3 = P[3];
            const float4 w0 = mat_col(p0, p1, p2, p3, C[0]), w1 = mat_col(p0, p1, p2, p3, C[1]);
            const float4 w2 = mat_col(p0, p1, p2, p3, C[2]), w3 = mat_col(p0, p1, p2, p3, C[3]);
            C[0] = w0;
            C[1] = w1;
            C[2] = w2;
            C[3] = w3;
            st_f8(world + 4 * (size_t)i, w0, w1);
            st_f8(world + 4 * (size_t)i + 2, w2, w3);
        }
        __syncthreads();
        prev = m;
        np = n;
        m += n;
        po += pad16_words(n);
    }
}

}  // namespace

cudaError_t launch_small_levels(const FoldArgs& a, cudaStream_t stream)
{
    uint32_t total = a.n0;
    for (uint32_t l = 0; l < a.count; l++) total += a.lvl[l].n;
    if (total > kFoldMaxNodes || a.count == 0 || a.count >= CADR_MAX_LEVELS) return cudaErrorInvalidValue;
    propagate_small_levels_kernel<<<1, kFoldThreads, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_propagate(const float4* parent_world, uint32_t num_parents, const float4* local,
                             const uint32_t* parent, uint32_t n, float4* world, int staged,
                             uint32_t* error, uint64_t spin_limit_ns, cudaStream_t stream,
                             bool after_level_kernel)
{
    if (n == 0) return cudaSuccess;
    const uint32_t grid = (n + kPropThreads - 1) / kPropThreads;
    if (!after_level_kernel) {
        propagate_kernel<<<grid, kPropThreads, 0, stream>>>(parent_world, num_parents, local, parent, n,
                                                            world, staged, error, spin_limit_ns);
        return cudaGetLastError();
    }
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cf = {};
    cf.gridDim = dim3(grid);
    cf.blockDim = dim3(kPropThreads);
    cf.stream = stream;
    cf.attrs = &at;
    cf.numAttrs = 1;
    return cudaLaunchKernelEx(&cf, propagate_kernel, parent_world, num_parents, local, parent, n, world, staged,
                              error, spin_limit_ns);
}

cudaError_t launch_leaf_propagate(const LeafArgs& a, cudaStream_t stream)
{
    if (a.n == 0) return cudaSuccess;
    const uint32_t grid = (a.n + kLeafTile - 1) / kLeafTile;
    leaf_propagate_kernel<<<grid, kLeafThreads, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_leaf_stream_scan(const LeafArgs& a, Scratch& s, cudaStream_t stream, cudaEvent_t after_stream,
                                    bool after_level_kernel)
{
    if (a.n == 0) return cudaSuccess;
    const uint32_t tiles = (a.n + kLeafTile - 1) / kLeafTile;
    LeafArgs b = a;
    b.planes = s.planes;
    b.tile_words = reinterpret_cast<uint32_t*>(s.tile_state);
    if (after_level_kernel) {
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at.val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cf = {};
        cf.gridDim = dim3(tiles);
        cf.blockDim = dim3(kLeafThreads);
        cf.stream = stream;
        cf.attrs = &at;
        cf.numAttrs = 1;
        const cudaError_t el = cudaLaunchKernelEx(&cf, leaf_stream_kernel, b);
        if (el != cudaSuccess) return el;
    } else {
        leaf_stream_kernel<<<tiles, kLeafThreads, 0, stream>>>(b);
    }
    if (after_stream) {
        const cudaError_t er = cudaEventRecord(after_stream, stream);
        if (er != cudaSuccess) return er;
    }
    leaf_tile_scan_kernel<<<1, kScanThreads, 0, stream>>>(b.tile_words, tiles);
    return cudaGetLastError();
}

cudaError_t launch_leaf_region_counts(const LeafArgs& a, Scratch& s, cudaStream_t stream)
{
    if (a.num_state_sets == 0) return cudaSuccess;
    const uint32_t grid = (a.num_state_sets + 7) / 8;
    leaf_region_count_kernel<<<grid, 256, 0, stream>>>(s.planes, reinterpret_cast<const uint32_t*>(s.tile_state),
                                                       a.offsets, a.num_state_sets, a.counts);
    return cudaGetLastError();
}

cudaError_t launch_leaf_write(const LeafArgs& a, Scratch& s, cudaStream_t stream, bool after_scan)
{
    if (a.n == 0) return cudaSuccess;
    const uint32_t tiles = (a.n + kLeafTile - 1) / kLeafTile;
    LeafArgs c = a;
    c.planes = s.planes;
    c.tile_words = reinterpret_cast<uint32_t*>(s.tile_state);
    c.off_cap = kWriteOffsetCap;
    const size_t smem = ((a.num_state_sets + 1 <= kWriteOffsetCap) ? a.num_state_sets + 1 : 0) * sizeof(uint32_t);
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(tiles);
    cfg.blockDim = dim3(kLeafThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = after_scan ? &attr : nullptr;
    cfg.numAttrs = after_scan ? 1 : 0;
    const cudaError_t e = c.shard.dst_base ? cudaLaunchKernelEx(&cfg, leaf_write_kernel<true>, c)
                                           : cudaLaunchKernelEx(&cfg, leaf_write_kernel<false>, c);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t launch_leaf_cull(const LeafArgs& a, Scratch& s, cudaStream_t stream, cudaEvent_t after_stream,
                             bool after_level_kernel)
{
    if (a.n == 0) return cudaSuccess;
    const cudaError_t e = launch_leaf_stream_scan(a, s, stream, after_stream, after_level_kernel);
    if (e != cudaSuccess) return e;
    LeafArgs c = a;
    c.shard = ShardPlacement{};
    return launch_leaf_write(c, s, stream, true);
}

}  // namespace cadr
