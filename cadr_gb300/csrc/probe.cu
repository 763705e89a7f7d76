// probe.cu - the bandwidth a plain pass's leaf stream can reach on this
// GPU: a kernel that moves the same traffic (per drawable 64 B local
// matrix + 16 B sphere + 4 B parent index read, 64 B world matrix written)
// with the same access pattern (per-lane 64-byte records, world matrices
// leaving through a swizzled per-warp block) and no arithmetic.  A
// measurement aid for the roofline of the stream kernel.
#include "capi_internal.h"

namespace cadr {

namespace {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) stream_mix_kernel(const float4* __restrict__ local,
                                                                  const float4* __restrict__ sphere,
                                                                  const uint32_t* __restrict__ parent,
                                                                  float4* __restrict__ world, uint32_t n,
                                                                  uint32_t* sink)
{
    __shared__ float4 xb[kProbeThreads / kWarp][4 * kWarp];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t i0 = blockIdx.x * (uint32_t)kProbeThreads + warp * (uint32_t)kWarp;
    if (i0 >= n) return;
    const uint32_t i = i0 + lane;
    const uint32_t cnt = min((uint32_t)kWarp, n - i0);
    float4* b = xb[warp];
    if (i < n) {
        float4 c0, c1, c2, c3;
        ld_nc_f8(local + (size_t)i * 4, c0, c1);
        ld_nc_f8(local + (size_t)i * 4 + 2, c2, c3);
        const float4 sp = ld_nc_f4(sphere + i);
        const uint32_t p = ld_nc_u32(parent + i);
        // Keeps the sphere and parent loads (never true for the probe's
        // zero-filled inputs).
        if (p == 0xffffffffu && sp.w == -1.0f) atomicOr(sink, 1u);
        const uint32_t q = 4u * lane;
        b[(q + 0) ^ (((q + 0) >> 3) & 3u)] = c0;
        b[(q + 1) ^ (((q + 1) >> 3) & 3u)] = c1;
        b[(q + 2) ^ (((q + 2) >> 3) & 3u)] = c2;
        b[(q + 3) ^ (((q + 3) >> 3) & 3u)] = c3;
    }
    __syncwarp();
    float4* wp = world + (size_t)i0 * 4;
#pragma unroll
    for (uint32_t k = 0; k < 4; k++) {
        const uint32_t q = lane + 32u * k;
        if ((q >> 2) < cnt) st_cs_f4(wp + q, b[q ^ ((q >> 3) & 3u)]);
    }
}

}  // namespace

}  // namespace cadr

using namespace cadr;

extern "C" {

CADR_API cadr_status cadr_measure_stream_mix(cadr_context* ctx, uint64_t num_drawables, uint32_t reps,
                                             double* gbytes_per_s)
{
    if (!ctx || !gbytes_per_s || num_drawables == 0 || num_drawables > 0xffffffffull || reps == 0)
        return fail(CADR_ERR_INVALID_ARG, "measure_stream_mix: bad argument");
    DeviceGuard dg(ctx->device);
    const uint64_t n = num_drawables;
    const size_t bytes = (size_t)n * (64 + 16 + 4 + 64) + 3 * 256 + 4;
    cudaStream_t s = ctx->stream;
    uint8_t* base = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&base), bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "measure_stream_mix: device memory");
    auto align = [](size_t o) { return (o + 255) & ~size_t(255); };
    const size_t o_sphere = align(n * 64), o_parent = align(o_sphere + n * 16), o_world = align(o_parent + n * 4),
                 o_sink = o_world + n * 64;
    const float4* local = reinterpret_cast<const float4*>(base);
    const float4* sphere = reinterpret_cast<const float4*>(base + o_sphere);
    const uint32_t* parent = reinterpret_cast<const uint32_t*>(base + o_parent);
    float4* world = reinterpret_cast<float4*>(base + o_world);
    uint32_t* sink = reinterpret_cast<uint32_t*>(base + o_sink);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMemsetAsync(base, 0, o_world, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sink, 0, 4, s);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const uint32_t grid = (uint32_t)((n + kProbeThreads - 1) / kProbeThreads);
    for (uint32_t k = 0; e == cudaSuccess && k < reps + 2; k++) {
        if (k == 2) e = cudaEventRecord(e0, s);
        if (e != cudaSuccess) break;
        stream_mix_kernel<<<grid, kProbeThreads, 0, s>>>(local, sphere, parent, world, (uint32_t)n, sink);
        e = cudaGetLastError();
        if (e == cudaSuccess) ctx->launches++;
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    const cudaError_t ef = cudaFreeAsync(base, s);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "measure_stream_mix");
    *gbytes_per_s = (double)reps * (double)n * 148.0 / (ms * 1e-3) / 1e9;
    return CADR_OK;
}

}  // extern "C"
