// tier_a.cu - the handle-resolution pass of the reference's
// processDrawables compute shader (src/CadR/shaders/processDrawables.comp:92-113),
// one thread per drawable instead of one 1-invocation workgroup.
//
// Per drawable i (records packed in StateSet depth-first order):
//   ps = lookup(primitiveSetHandle) + primitiveSetOffset
//   ml = lookup(matrixListHandle)
//   indirect[i] = {ps.count, ml.numMatrices, ps.first, 0}
//   pointers[i] = {lookup(vertexDataHandle), lookup(indexDataHandle), ml,
//                  lookup(drawableDataHandle)}
// lookup() is the 1/2/3-level table walk of processDrawables.comp:77-89,
// with the same 32-bit truncations.  The 48-byte record is read as three
// 16-byte vectors; the five lookups are independent chains, so their loads
// overlap; the 16- and 32-byte outputs are written as 16-byte vectors.
#include "handles.cuh"
#include "kernels.cuh"

namespace cadr {

namespace {

template <int LEVEL>
__global__ void __launch_bounds__(256) process_drawables_kernel(
    const uint64_t* __restrict__ root, const ulonglong2* __restrict__ drawables, uint64_t n,
    uint4* __restrict__ indirect, ulonglong2* __restrict__ pointers)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ulonglong2* d = drawables + i * 3;
    const ulonglong2 d0 = __ldg(d + 0);  // vertexDataHandle, indexDataHandle
    const ulonglong2 d1 = __ldg(d + 1);  // matrixListHandle, drawableDataHandle
    const ulonglong2 d2 = __ldg(d + 2);  // primitiveSetHandle, primitiveSetOffset | padding
    uint4 ind;
    ulonglong2 p0, p1;
    resolve_record<LEVEL>(root, d0, d1, d2, ind, p0, p1);
    indirect[i] = ind;
    pointers[i * 2 + 0] = p0;
    pointers[i * 2 + 1] = p1;
}

}  // namespace

cudaError_t launch_process_drawables(uint32_t level, const uint64_t* root,
                                     const cadr_drawable_gpu_data* drawables, uint64_t n,
                                     cadr_draw_indirect_cmd* indirect,
                                     cadr_drawable_pointers* pointers, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    const uint64_t grid = (n + 255) / 256;
    auto d = reinterpret_cast<const ulonglong2*>(drawables);
    auto ind = reinterpret_cast<uint4*>(indirect);
    auto ptr = reinterpret_cast<ulonglong2*>(pointers);
    switch (level) {
    case 1: process_drawables_kernel<1><<<(unsigned)grid, 256, 0, stream>>>(root, d, n, ind, ptr); break;
    case 2: process_drawables_kernel<2><<<(unsigned)grid, 256, 0, stream>>>(root, d, n, ind, ptr); break;
    default: process_drawables_kernel<3><<<(unsigned)grid, 256, 0, stream>>>(root, d, n, ind, ptr); break;
    }
    return cudaGetLastError();
}

}  // namespace cadr
