// consumer.cu - vertex-pulling consumer check of the Tier A draws.
//
// The draws that cadr_process_drawables writes are consumed by a vertex
// shader that pulls its inputs through the DrawablePointers
// (examples/RenderingPerformance/shader.vert:100-120): the index at
// gl_VertexIndex from the index buffer, the position at that index from
// the vertex buffer, the model matrix at gl_InstanceIndex from the matrix
// list.  This kernel makes the same reads for every vertex of every draw,
// in CUDA, after checking each address against the memory the draws may
// address, and hashes the transformed positions, so that a whole frame's
// draw buffers can be verified against the oracle without a graphics API.
#include <algorithm>

#include "capi_internal.h"

using namespace cadr;

namespace cadr {
namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;
constexpr int kCheckThreads = 256;

struct Regions {
    uint64_t base[CADR_MAX_MEMORY_REGIONS];
    uint64_t end[CADR_MAX_MEMORY_REGIONS];
    uint32_t count;
};

// [addr, addr + bytes) lies in one region and addr is a multiple of align.
__device__ __forceinline__ bool readable(const Regions& r, uint64_t addr, uint64_t bytes, uint64_t align)
{
    if (addr % align) return false;
    for (uint32_t k = 0; k < r.count; k++)
        if (addr >= r.base[k] && addr <= r.end[k] && bytes <= r.end[k] - addr) return true;
    return false;
}

// SplitMix64 finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom
// number generators", 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t pair(float lo, float hi)
{
    return (uint64_t)__float_as_uint(lo) | ((uint64_t)__float_as_uint(hi) << 32);
}

__device__ __forceinline__ float4 ld_f4(const void* p) { return *reinterpret_cast<const float4*>(p); }

// One warp per draw, the warps striding over the draws.
__global__ void __launch_bounds__(kCheckThreads) check_draws_kernel(const cadr_draw_indirect_cmd* __restrict__ indirect,
                                                                    const cadr_drawable_pointers* __restrict__ pointers,
                                                                    uint64_t n, const Regions reg,
                                                                    const cadr_consumer_view v,
                                                                    cadr_draw_check* __restrict__ out)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCheckThreads / 32);
    const float4 V0 = make_float4(v.view[0], v.view[1], v.view[2], v.view[3]);
    const float4 V1 = make_float4(v.view[4], v.view[5], v.view[6], v.view[7]);
    const float4 V2 = make_float4(v.view[8], v.view[9], v.view[10], v.view[11]);
    const float4 V3 = make_float4(v.view[12], v.view[13], v.view[14], v.view[15]);
    for (uint64_t d = (uint64_t)blockIdx.x * (kCheckThreads / 32) + (threadIdx.x >> 5); d < n; d += warps) {
        const cadr_draw_indirect_cmd cmd = indirect[d];
        const cadr_drawable_pointers dp = pointers[d];
        uint32_t flags = 0, pulled = 0;
        uint64_t sum = 0;
        if (dp.drawable_data_ptr && !readable(reg, dp.drawable_data_ptr, 64, 64)) flags |= CADR_DRAW_BAD_DRAWABLE_DATA;
        const uint64_t ml = dp.matrix_list_ptr;
        if (!readable(reg, ml, 64, 64)) {
            flags |= CADR_DRAW_BAD_MATRIX_LIST;
        } else {
            const uint32_t num_matrices = *reinterpret_cast<const uint32_t*>(ml);
            for (uint64_t m = cmd.first_instance; m < (uint64_t)cmd.first_instance + cmd.instance_count; m++) {
                const uint64_t ma = ml + 64 + 64 * m;
                if (m >= num_matrices) {  // and so are all later instances
                    flags |= CADR_DRAW_BAD_INSTANCE;
                    break;
                }
                if (!readable(reg, ma, 64, 16)) {
                    flags |= CADR_DRAW_BAD_MATRIX_LIST;
                    continue;
                }
                const float4 M0 = ld_f4(reinterpret_cast<const void*>(ma)), M1 = ld_f4(reinterpret_cast<const void*>(ma + 16));
                const float4 M2 = ld_f4(reinterpret_cast<const void*>(ma + 32)), M3 = ld_f4(reinterpret_cast<const void*>(ma + 48));
                // modelViewMatrix = scene.viewMatrix * matrices[gl_InstanceIndex]
                const float4 W0 = mat_col(V0, V1, V2, V3, M0), W1 = mat_col(V0, V1, V2, V3, M1);
                const float4 W2 = mat_col(V0, V1, V2, V3, M2), W3 = mat_col(V0, V1, V2, V3, M3);
                for (uint64_t k = lane; k < cmd.vertex_count; k += 32) {
                    const uint64_t ia = dp.index_data_ptr + 4ull * ((uint64_t)cmd.first_vertex + k);
                    if (!readable(reg, ia, 4, 4)) {  // the lane's later indices follow it in memory
                        flags |= CADR_DRAW_BAD_INDEX_READ;
                        break;
                    }
                    const uint32_t index = *reinterpret_cast<const uint32_t*>(ia);
                    const uint64_t va = dp.vertex_data_ptr + 12ull * index;
                    if (!readable(reg, va, 12, 4)) {
                        flags |= CADR_DRAW_BAD_VERTEX_READ;
                        continue;
                    }
                    const float* p = reinterpret_cast<const float*>(va);
                    const float4 eye = mat_col(W0, W1, W2, W3, make_float4(p[0], p[1], p[2], 1.0f));
                    const float gx = fadd(fadd(fmul(v.p11, eye.x), fmul(v.p31, eye.z)), fmul(v.p41, eye.w));
                    const float gy = fadd(fadd(fmul(v.p22, eye.y), fmul(v.p32, eye.z)), fmul(v.p42, eye.w));
                    const float gz = fadd(fmul(v.p33, eye.z), fmul(v.p43, eye.w));
                    const float gw = fadd(fmul(v.p34, eye.z), fmul(v.p44, eye.w));
                    const float ex = fdiv(eye.x, eye.w), ey = fdiv(eye.y, eye.w), ez = fdiv(eye.z, eye.w);
                    sum += mix64(pair(gx, gy)) ^ mix64(pair(gz, gw) ^ kGolden) ^ mix64(pair(ex, ey) ^ (2 * kGolden)) ^
                           mix64(((uint64_t)__float_as_uint(ez) | ((uint64_t)index << 32)) ^ (3 * kGolden));
                    pulled++;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum += __shfl_xor_sync(~0u, sum, o);
            pulled += __shfl_xor_sync(~0u, pulled, o);
            flags |= __shfl_xor_sync(~0u, flags, o);
        }
        if (lane == 0) {
            cadr_draw_check c;
            c.checksum = sum;
            c.pulled = pulled;
            c.flags = flags;
            out[d] = c;
        }
    }
}

}  // namespace
}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_check_draws(cadr_context* ctx, const cadr_draw_indirect_cmd* indirect,
                                      const cadr_drawable_pointers* pointers, uint64_t num_draws,
                                      const cadr_memory_region* regions, uint32_t num_regions,
                                      const cadr_consumer_view* view, cadr_draw_check* out, cadr_stream stream)
{
    if (!ctx || !view || (num_draws && (!indirect || !pointers || !out)) || (num_regions && !regions))
        return fail(CADR_ERR_INVALID_ARG, "check_draws: null argument");
    DeviceGuard dg(ctx->device);
    if (num_regions > CADR_MAX_MEMORY_REGIONS)
        return fail(CADR_ERR_INVALID_ARG, "check_draws: %u regions exceed %u", num_regions, CADR_MAX_MEMORY_REGIONS);
    if ((reinterpret_cast<uintptr_t>(indirect) | reinterpret_cast<uintptr_t>(out)) % 16 ||
        reinterpret_cast<uintptr_t>(pointers) % 32)
        return fail(CADR_ERR_INVALID_ARG, "check_draws: misaligned buffer");
    if (num_draws == 0) return CADR_OK;
    Regions r{};
    r.count = num_regions;
    for (uint32_t k = 0; k < num_regions; k++) {
        if (regions[k].size > ~0ull - regions[k].base)
            return fail(CADR_ERR_INVALID_ARG, "check_draws: region %u wraps the address space", k);
        r.base[k] = regions[k].base;
        r.end[k] = regions[k].base + regions[k].size;
    }
    cudaStream_t s = pick_stream(ctx, stream);
    const uint64_t want = (num_draws + (kCheckThreads / 32) - 1) / (kCheckThreads / 32);
    const uint32_t grid = (uint32_t)std::min<uint64_t>(want, (uint64_t)ctx->num_sms * 16);
    check_draws_kernel<<<grid, kCheckThreads, 0, s>>>(indirect, pointers, num_draws, r, *view, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "check_draws: launch");
    ctx->launches++;
    return CADR_OK;
}

}  // extern "C"
