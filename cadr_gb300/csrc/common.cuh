// common.cuh - device helpers shared by the kernels of libcadr_cuda.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cadr_cuda.h"
#include "fp.cuh"

namespace cadr {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Lookback control block: one per scratch area (one per concurrently
// running pass).  The last CTA of a pass resets the tile counter and bumps
// the epoch, so the next pass (or the next replay of a captured graph)
// starts clean without a memset.
struct LookbackCtl {
    uint32_t tile_counter;
    uint32_t done_counter;
    uint32_t epoch;
    uint32_t pad;
};

// Tile status word: [63..35] epoch (29 bits) | [34..33] status | [32] head
// flag | [31..0] value.  status 0 = not published, 1 = aggregate, 2 = prefix.
// `head` marks a tile that contains the start of a StateSet region: its
// value then counts only from the last region start, and a lookback may
// stop there (segmented scan).
constexpr uint64_t kStatusAgg = 1, kStatusPrefix = 2;
constexpr uint32_t kEpochMask = 0x1fffffffu;

__device__ __forceinline__ uint64_t pack_status(uint32_t epoch, uint64_t status, uint32_t head,
                                                uint32_t value)
{
    return ((uint64_t)(epoch & kEpochMask) << 35) | (status << 33) | ((uint64_t)(head & 1u) << 32) |
           (uint64_t)value;
}
__device__ __forceinline__ uint32_t st_epoch(uint64_t w) { return (uint32_t)(w >> 35); }
__device__ __forceinline__ uint32_t st_status(uint64_t w) { return (uint32_t)(w >> 33) & 3u; }
__device__ __forceinline__ uint32_t st_head(uint64_t w) { return (uint32_t)(w >> 32) & 1u; }
__device__ __forceinline__ uint32_t st_value(uint64_t w) { return (uint32_t)w; }

__device__ __forceinline__ void store_relaxed_u64(uint64_t* p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t load_relaxed_u64(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t load_relaxed_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// Streaming loads / stores.
__device__ __forceinline__ float4 ld_nc_f4(const float4* p)
{
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_nc_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_cs_f4(float4* p, float4 v)
{
    asm volatile("st.global.cs.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w)
                 : "memory");
}
// 256-bit forms (sm_100 and later): p must be 32-byte aligned.  One
// instruction moves two float4, halving the L1 requests of a per-lane
// 64-byte record.
__device__ __forceinline__ void ld_nc_f8(const float4* p, float4& a, float4& b)
{
    asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p));
}
__device__ __forceinline__ void st_f8(float4* p, float4 a, float4 b)
{
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(a.x), "f"(a.y),
                 "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}

// ---------------------------------------------------------------------------
// mbarrier + bulk (TMA) copy global -> shared, non-multicast, own CTA only.
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Retires an mbarrier before its shared memory is given back.
__device__ __forceinline__ void mbar_inval(uint64_t* bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Requires 16-byte aligned dst/src and bytes % 16 == 0.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Bulk (TMA) copy shared -> global, tracked by the issuing thread's bulk
// groups.  Requires 16-byte aligned dst/src and bytes % 16 == 0.
__device__ __forceinline__ void bulk_copy_s2g(void* dst, const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(smem_addr(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until all committed bulk groups of this thread have finished reading
// their shared-memory source (the buffer may be overwritten afterwards).
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Wait until all committed bulk groups of this thread are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) accesses of that memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Asynchronous 8-byte copy global -> shared (both 8-byte aligned), with no
// register holding the value; cp_async_wait_all() waits for this thread's
// copies.
__device__ __forceinline__ void cp_async_8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bulk (TMA) prefetch of [src, src + bytes) into L2; 16-byte aligned
// address, bytes % 16 == 0.  Brings a whole tile's stream on its way with
// one instruction and no registers.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Programmatic dependent launch.  A kernel launched with programmatic
// stream serialization may start before the kernel ahead of it on the
// stream has finished; grid_dependency_wait() returns when that kernel has
// completed and its memory writes are visible.  grid_dependents_launch()
// lets the next such kernel start now.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dependents_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Bounded wait on phase `parity`; returns false (after limit_ns) when the
// barrier never completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < (1u << 30); it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && global_timer_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Where a shard of a pass split over several devices puts its commands:
// the k-th visible drawable of StateSet region s goes to dst_base[s] + k of
// a merged buffer of `capacity` commands, with firstInstance = its index in
// the shard + first_instance (its index in the whole scene).
struct ShardPlacement {
    const uint32_t* dst_base;
    uint32_t first_instance;
    uint32_t capacity;
};

// ---------------------------------------------------------------------------
// View constants as the kernels consume them.
struct ViewConst {
    float4 plane[6];
    float4 view_z;
    float4 lod_threshold;
    float lod_scale;
    float near_z;
    uint32_t perspective;
    uint32_t pad;
};
static_assert(sizeof(ViewConst) == sizeof(cadr_view), "view layout");

// GLM-order 4x4 product (column-major): r[c] = ((a0*b[c].x + a1*b[c].y) + a2*b[c].z) + a3*b[c].w
__device__ __forceinline__ float4 mat_col(const float4 a0, const float4 a1, const float4 a2,
                                          const float4 a3, const float4 b)
{
    float4 r;
    r.x = fadd(fadd(fadd(fmul(a0.x, b.x), fmul(a1.x, b.y)), fmul(a2.x, b.z)), fmul(a3.x, b.w));
    r.y = fadd(fadd(fadd(fmul(a0.y, b.x), fmul(a1.y, b.y)), fmul(a2.y, b.z)), fmul(a3.y, b.w));
    r.z = fadd(fadd(fadd(fmul(a0.z, b.x), fmul(a1.z, b.y)), fmul(a2.z, b.z)), fmul(a3.z, b.w));
    r.w = fadd(fadd(fadd(fmul(a0.w, b.x), fmul(a1.w, b.y)), fmul(a2.w, b.z)), fmul(a3.w, b.w));
    return r;
}

// BoundingSphere operator* (src/CadR/BoundingSphere.h:70-86).
__device__ __forceinline__ float4 transform_sphere(const float4 m0, const float4 m1, const float4 m2,
                                                   const float4 m3, const float4 s)
{
    float4 o;
    o.x = fadd(fadd(fadd(fmul(m0.x, s.x), fmul(m1.x, s.y)), fmul(m2.x, s.z)), m3.x);
    o.y = fadd(fadd(fadd(fmul(m0.y, s.x), fmul(m1.y, s.y)), fmul(m2.y, s.z)), m3.y);
    o.z = fadd(fadd(fadd(fmul(m0.z, s.x), fmul(m1.z, s.y)), fmul(m2.z, s.z)), m3.z);
    const float l0 = fadd(fadd(fmul(m0.x, m0.x), fmul(m0.y, m0.y)), fmul(m0.z, m0.z));
    const float l1 = fadd(fadd(fmul(m1.x, m1.x), fmul(m1.y, m1.y)), fmul(m1.z, m1.z));
    const float l2 = fadd(fadd(fmul(m2.x, m2.x), fmul(m2.y, m2.y)), fmul(m2.z, m2.z));
    float mx = (l0 < l1) ? l1 : l0;
    mx = (mx < l2) ? l2 : mx;
    o.w = sphere_radius(mx, s.w);
    return o;
}

// Plane test, marginal band and LOD (same spec as the oracle's classify).
// A sphere is marginal when its surface lies within kMarginalBand of a
// plane: |dist + r| <= 1e-5, in world units.
constexpr float kMarginalBand = 1e-5f;

__device__ __forceinline__ void classify(const ViewConst& v, const float4 ws, uint32_t num_lods,
                                         bool& visible, bool& marginal, uint32_t& lod)
{
    bool vis = true, mar = false;
    const float nr = -ws.w;
#pragma unroll
    for (int p = 0; p < 6; p++) {
        const float4 pl = v.plane[p];
        const float dist = fadd(fadd(fadd(fmul(pl.x, ws.x), fmul(pl.y, ws.y)), fmul(pl.z, ws.z)), pl.w);
        // bitwise, not short-circuit: every plane test runs, branch-free
        vis &= (dist >= nr);
        mar |= (fabsf(fadd(dist, ws.w)) <= kMarginalBand);
    }
    float zc = 1.0f;
    if (v.perspective) {
        const float z = fadd(fadd(fadd(fmul(v.view_z.x, ws.x), fmul(v.view_z.y, ws.y)),
                                  fmul(v.view_z.z, ws.z)),
                             v.view_z.w);
        zc = fmaxf(-z, v.near_z);
    }
    const float s = fmul(ws.w, v.lod_scale);
    uint32_t l = num_lods - 1;
    const float th[3] = {v.lod_threshold.x, v.lod_threshold.y, v.lod_threshold.z};
#pragma unroll
    for (int k = 2; k >= 0; k--)
        if (((uint32_t)k + 1 < num_lods) & (s >= fmul(th[k], zc))) l = (uint32_t)k;
    visible = vis;
    marginal = mar;
    lod = l;
}

// Internal-consistency checks.  In the bounds-checked build (CADR_BOUNDS_CHECK
// defined) CADR_CHECKED(cond, error) evaluates cond, records
// CADR_DEVERR_BOUNDS in *error when it is false and returns it, so that the
// access it guards is skipped; in the product build it is the constant true
// and cond is not evaluated.  It guards indices that the kernels derive
// themselves (slots, plane words, work items); indices read from the
// caller's data are checked in every build (CADR_DEVERR_BAD_INDEX).
#ifdef CADR_BOUNDS_CHECK
__device__ __forceinline__ bool bounds_checked(bool ok, uint32_t* error)
{
    if (!ok) atomicOr(error, CADR_DEVERR_BOUNDS);
    return ok;
}
#define CADR_CHECKED(cond, error) (::cadr::bounds_checked((cond), (error)))
#else
#define CADR_CHECKED(cond, error) true
#endif

// Whether position i and its command slot both lie in region r.
__device__ __forceinline__ bool in_region(const uint32_t* offsets, uint32_t r, uint32_t i, uint32_t slot)
{
    const uint32_t s = offsets[r], e = offsets[r + 1];
    return s <= i && i < e && s <= slot && slot < e;
}

// First index s in [lo, hi) with offsets[s] > key, minus one: the region
// that contains position `key` (regions may be empty).  `offsets` may point
// to global or (staged) shared memory.
__device__ __forceinline__ uint32_t region_of(const uint32_t* offsets, uint32_t lo, uint32_t hi, uint32_t key)
{
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offsets[mid] <= key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo - 1;
}

// region_of(offsets, 0, S + 1, key) by a whole warp (every lane returns
// it): a 32-way search, two rounds up to 1,024 entries.  offsets[0] is 0,
// so the answer is at least 0.
__device__ __forceinline__ uint32_t warp_region_of(const uint32_t* offsets, uint32_t S, uint32_t key)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lo = 0, hi = S + 1;  // the answer is in [lo, hi); offsets[lo] <= key
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31u) / 32u;
        const uint32_t k = lo + lane * step;
        const uint32_t m = __ballot_sync(~0u, k < hi && offsets[k] <= key);
        lo += (31u - (uint32_t)__clz(m)) * step;  // lane 0 always holds
        hi = min(hi, lo + step);
    }
    return lo;
}

// Stages the S+1 StateSet offsets into shared memory when they fit `cap`
// entries (all threads of the CTA call it; the caller's next
// __syncthreads() publishes them) and returns the array to search.
__device__ __forceinline__ const uint32_t* stage_offsets(uint32_t* smem, uint32_t cap, const uint32_t* offsets,
                                                         uint32_t S)
{
    if (S + 1 > cap) return offsets;
    for (uint32_t k = threadIdx.x; k <= S; k += blockDim.x) smem[k] = __ldg(offsets + k);
    return smem;
}

}  // namespace cadr
