// leaf_tma.cu - the fused leaf pass with its streams moved by TMA.
//
// Each CTA takes the next tile of 512 drawables from the tile counter and,
// from one thread, issues four bulk (TMA) copies global -> shared of the
// tile's local matrices, spheres, geometry and parent indices (44 KiB),
// completed on an mbarrier: the loads in flight cost no registers, and the
// four CTAs resident on an SM (64 registers per thread) sit in different
// phases, so one CTA's copies overlap another's arithmetic and lookback.
// World matrices overwrite the local matrices in shared memory and leave
// with one bulk copy shared -> global.  Parent world matrices are gathered
// from L2 before any arithmetic.  Compaction is the segmented decoupled
// lookback of compact.cuh and the arithmetic is leaf_kernel's, so results
// are bit-identical.
//
// Shared-memory reads of the 64-byte matrix records are conflict-free: at
// step k thread t handles column (k + (t >> 1)) & 3, which spreads every
// quarter-warp over eight distinct 16-byte bank groups.
#include <algorithm>

#include "compact.cuh"
#include "kernels.cuh"

namespace cadr {

namespace {

constexpr int kTT = 256;          // threads per CTA
constexpr int kTI = 2;            // drawables per thread and tile
constexpr int kTS = kTT * kTI;    // drawables per tile
using TmaTile = Tile<kTT, kTI>;

struct __align__(128) TmaSmem {
    float4 mat[kTS * 4];  // local matrices in, world matrices out (32 KiB)
    float4 sph[kTS];      // 8 KiB
    uint32_t geo[kTS];    // 2 KiB
    uint32_t par[kTS];    // 2 KiB
    TmaTile::Smem tile;
    uint64_t bar;
    uint32_t skip;
};

__global__ void __launch_bounds__(kTT, 4) leaf_tma_kernel(const LeafArgs a, const Scratch s)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TmaSmem& sm = *reinterpret_cast<TmaSmem*>(smem_raw);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

    if (t == 0) {
        const uint32_t tile = atomicAdd(&s.ctl->tile_counter, 1u);
        sm.tile.info[0] = tile;
        sm.tile.info[1] = load_relaxed_u32(&s.ctl->epoch);
        // A tile number past the scene (only if the control block was not
        // re-armed) touches nothing but the completion counter.
        sm.skip = (uint64_t)tile * (uint64_t)kTS >= (uint64_t)a.n;
        if (!sm.skip) {
            const uint32_t b = tile * (uint32_t)kTS;
            const uint32_t rows = min((uint32_t)kTS, a.n - b);
            const uint32_t r16 = (rows * 4u + 15u) & ~15u;  // 4-byte arrays, rounded up to 16 bytes
            mbar_init(&sm.bar, 1);
            mbar_arrive_expect_tx(&sm.bar, rows * 64u + rows * 16u + r16 + (a.parent ? r16 : 0u));
            bulk_copy_g2s(sm.mat, a.local + (size_t)b * 4, rows * 64u, &sm.bar);
            bulk_copy_g2s(sm.sph, a.sphere + b, rows * 16u, &sm.bar);
            bulk_copy_g2s(sm.geo, a.geometry + b, r16, &sm.bar);
            if (a.parent) bulk_copy_g2s(sm.par, a.parent + b, r16, &sm.bar);
        }
    }
    __syncthreads();
    if (sm.skip) {
        if (t == 0) finish_pass(s.ctl);
        return;
    }
    const uint32_t tile = sm.tile.info[0];
    const uint32_t b = tile * (uint32_t)kTS;
    if (!mbar_wait_bounded(&sm.bar, 0, a.spin_limit_ns) && t == 0)
        atomicOr(a.error, CADR_DEVERR_MBARRIER_TIMEOUT);

    float4 P[kTI][4];
    uint32_t geo[kTI];
#pragma unroll
    for (int j = 0; j < kTI; j++) {
        const uint32_t q = (uint32_t)(j * kTT + t);
        const bool valid = b + q < a.n;
        geo[j] = valid ? sm.geo[q] : 0u;
        if (valid && a.parent) {
            uint32_t p = sm.par[q];
            if (p >= a.num_parents) {
                atomicOr(a.error, CADR_DEVERR_BAD_INDEX);
                p = 0;
            }
            const float4* pp = a.parent_world + (size_t)p * 4;
            P[j][0] = __ldg(pp);
            P[j][1] = __ldg(pp + 1);
            P[j][2] = __ldg(pp + 2);
            P[j][3] = __ldg(pp + 3);
        }
    }
    const uint32_t rot = ((uint32_t)t >> 1) & 3u;
    uint32_t vis_bits = 0, lod_bits = 0;
#pragma unroll
    for (int j = 0; j < kTI; j++) {
        const uint32_t q = (uint32_t)(j * kTT + t);
        const uint32_t i = b + q;
        bool visible = false, marginal = false;
        uint32_t lod = 0;
        if (i < a.n) {
            float4 w0, w1, w2, w3;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t c = ((uint32_t)k + rot) & 3u;
                const float4 l = sm.mat[q * 4 + c];
                const float4 w = a.parent ? mat_col(P[j][0], P[j][1], P[j][2], P[j][3], l) : l;
                sm.mat[q * 4 + c] = w;
                if (c == 0) w0 = w;
                else if (c == 1) w1 = w;
                else if (c == 2) w2 = w;
                else w3 = w;
            }
            const float4 ws = transform_sphere(w0, w1, w2, w3, sm.sph[q]);
            classify(a.view, ws, a.num_lods, visible, marginal, lod);
        }
        const uint32_t vb = __ballot_sync(~0u, visible);
        const uint32_t mb = __ballot_sync(~0u, marginal);
        const uint32_t word0 = b + (uint32_t)(j * kTT + warp * kWarp);
        if (lane == 0) {
            sm.tile.ballot[j][warp] = vb;
            if (a.marginal && word0 < a.n) a.marginal[word0 >> 5] = mb;
        }
        vis_bits |= (visible ? 1u : 0u) << j;
        lod_bits |= lod << (2 * j);
    }
    // World matrices leave with one bulk copy.
    fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) {
        bulk_copy_s2g(a.world + (size_t)b * 4, sm.mat, min((uint32_t)kTS, a.n - b) * 64u);
        bulk_commit();
    }
    TmaTile::scan(sm.tile, a.offsets, a.num_state_sets, b, a.n);
    TmaTile::lookback(sm.tile, s.tile_state, tile, 0, a.offsets, b, a.spin_limit_ns, a.fault, a.error);
    TmaTile::write(sm.tile, vis_bits, lod_bits, geo, b, a.n, tile == 0, a.offsets, a.num_state_sets, a.lods,
                   a.num_geometries, a.num_lods, a.cmds, a.counts, a.error);
    if (t == 0) {
        bulk_wait_all();  // the store reads shared memory the next CTA will own
        mbar_inval(&sm.bar);
        finish_pass(s.ctl);
    }
}

bool g_attr_set[64] = {};

}  // namespace

uint32_t leaf_tma_tile() { return (uint32_t)kTS; }

cudaError_t launch_leaf_cull_tma(const LeafArgs& a, Scratch& s, int num_sms, int device, cudaStream_t stream)
{
    (void)num_sms;
    if (a.n == 0) return cudaSuccess;
    const uint32_t tiles = (a.n + kTS - 1) / kTS;
    const size_t smem = sizeof(TmaSmem);
    if (device >= 0 && device < 64 && !g_attr_set[device]) {
        cudaError_t e = cudaFuncSetAttribute(leaf_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        g_attr_set[device] = true;
    }
    leaf_tma_kernel<<<tiles, kTT, smem, stream>>>(a, s);
    return cudaGetLastError();
}

}  // namespace cadr
