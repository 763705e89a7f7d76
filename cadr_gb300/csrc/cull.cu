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

template <bool kCull>
__global__ void __launch_bounds__(kLeafThreads, 4) leaf_kernel(const LeafArgs a, const Scratch s)
{
    __shared__ LeafTile::Smem sm;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t tile;
    if (kCull) {
        if (t == 0) {
            sm.info[0] = atomicAdd(&s.ctl->tile_counter, 1u);
            sm.info[1] = load_relaxed_u32(&s.ctl->epoch);
        }
        __syncthreads();
        tile = sm.info[0];
    } else {
        tile = blockIdx.x;
    }
    // A tile number past the scene (only if the control block was not
    // re-armed) touches nothing but the completion counter.
    if ((uint64_t)tile * (uint64_t)kLeafTile >= (uint64_t)a.n) {
        if (kCull && t == 0) finish_pass(s.ctl);
        return;
    }
    const uint32_t b = tile * (uint32_t)kLeafTile;
    extern __shared__ uint32_t s_offsets[];
    const uint32_t* off = kCull ? stage_offsets(s_offsets, a.off_cap, a.offsets, a.num_state_sets) : a.offsets;

    uint32_t vis_bits = 0, lod_bits = 0;
    uint32_t geo[kLeafIpt];
#pragma unroll
    for (int j = 0; j < kLeafIpt; j++) {
        const uint32_t i = b + (uint32_t)(j * kLeafThreads + t);
        bool visible = false, marginal = false;
        uint32_t lod = 0;
        geo[j] = 0;
        if (i < a.n) {
            float4 l0, l1, l2, l3, w0, w1, w2, w3;
            load_mat(a.local + (size_t)i * 4, l0, l1, l2, l3);
            const float4 sp = ld_nc_f4(a.sphere + i);
            if (kCull) geo[j] = ld_nc_u32(a.geometry + i);
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
            float4* wp = a.world + (size_t)i * 4;
            st_cs_f4(wp + 0, w0);
            st_cs_f4(wp + 1, w1);
            st_cs_f4(wp + 2, w2);
            st_cs_f4(wp + 3, w3);
            const float4 ws = transform_sphere(w0, w1, w2, w3, sp);
            if (a.world_sphere) st_cs_f4(a.world_sphere + i, ws);
            if (kCull) classify(a.view, ws, a.num_lods, visible, marginal, lod);
        }
        if (kCull) {
            const uint32_t vb = __ballot_sync(~0u, visible);
            const uint32_t mb = __ballot_sync(~0u, marginal);
            const uint32_t word0 = b + (uint32_t)(j * kLeafThreads + warp * kWarp);
            if (lane == 0) {
                sm.ballot[j][warp] = vb;
                if (a.marginal && word0 < a.n) a.marginal[word0 >> 5] = mb;
            }
            vis_bits |= (visible ? 1u : 0u) << j;
            lod_bits |= lod << (2 * j);
        }
    }
    if (!kCull) return;
    __syncthreads();
    LeafTile::scan(sm, off, a.num_state_sets, b, a.n);
    LeafTile::lookback(sm, s.tile_state, tile, 0, off, b, a.spin_limit_ns, a.fault, a.error);
    LeafTile::write(sm, vis_bits, lod_bits, geo, b, a.n, tile == 0, off, a.num_state_sets, a.lods,
                    a.num_geometries, a.num_lods, a.cmds, a.counts, a.error);
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
    leaf_kernel<false><<<grid, kLeafThreads, 0, stream>>>(a, Scratch{});
    return cudaGetLastError();
}

// StateSet offsets are staged in shared memory up to this many entries.
constexpr uint32_t kLeafOffsetCap = 4096;

cudaError_t launch_leaf_cull(const LeafArgs& a, Scratch& s, cudaStream_t stream)
{
    if (a.n == 0) return cudaSuccess;
    const uint32_t grid = (a.n + kLeafTile - 1) / kLeafTile;
    LeafArgs b = a;
    b.off_cap = kLeafOffsetCap;
    const size_t smem = (a.num_state_sets + 1 <= kLeafOffsetCap) ? (a.num_state_sets + 1) * sizeof(uint32_t) : 0;
    leaf_kernel<true><<<grid, kLeafThreads, smem, stream>>>(b, s);
    return cudaGetLastError();
}

}  // namespace cadr
