// handles.cuh - the handle-table walk of the reference's processDrawables
// shader (src/CadR/shaders/processDrawables.comp:77-89) and the per-record
// resolution of :92-113, shared by the Tier A kernels.
#pragma once

#include <stdint.h>

namespace cadr {

__device__ __forceinline__ uint64_t ld_u64(uint64_t addr)
{
    return __ldg(reinterpret_cast<const unsigned long long*>(addr));
}

// t[uint(h)], t[uint(h>>11)][uint(h)&0x7ff] or
// t[uint(h>>22)][uint(h>>11)&0x7ff][uint(h)&0x7ff], with the shader's
// 32-bit truncations.
template <int LEVEL>
__device__ __forceinline__ uint64_t lookup(const uint64_t* __restrict__ root, uint64_t h)
{
    if (LEVEL == 1) return __ldg(reinterpret_cast<const unsigned long long*>(root) + (uint32_t)h);
    if (LEVEL == 2) {
        const uint64_t t2 = __ldg(reinterpret_cast<const unsigned long long*>(root) + (uint32_t)(h >> 11));
        return ld_u64(t2 + 8ull * ((uint32_t)h & 0x7ffu));
    }
    const uint64_t t2 = __ldg(reinterpret_cast<const unsigned long long*>(root) + (uint32_t)(h >> 22));
    const uint64_t t3 = ld_u64(t2 + 8ull * ((uint32_t)(h >> 11) & 0x7ffu));
    return ld_u64(t3 + 8ull * ((uint32_t)h & 0x7ffu));
}

// One record (three 16-byte words: vertex, index | matrix list, drawable
// data | primitive set, offset) to its indirect command and pointers:
//   ps = lookup(psH) + psOffset, ml = lookup(mlH)
//   indirect = {ps.count, ml.numMatrices, ps.first, 0}
//   pointers = {lookup(vertexH), lookup(indexH), ml, lookup(drawableDataH)}
// The five lookups are independent chains, so their loads overlap.
template <int LEVEL>
__device__ __forceinline__ void resolve_record(const uint64_t* __restrict__ root, const ulonglong2 d0,
                                               const ulonglong2 d1, const ulonglong2 d2, uint4& indirect,
                                               ulonglong2& p0, ulonglong2& p1)
{
    const uint64_t ps = lookup<LEVEL>(root, d2.x) + (uint64_t)(uint32_t)d2.y;
    const uint64_t ml = lookup<LEVEL>(root, d1.x);
    const uint64_t vtx = lookup<LEVEL>(root, d0.x);
    const uint64_t idx = lookup<LEVEL>(root, d0.y);
    const uint64_t dd = lookup<LEVEL>(root, d1.y);
    uint32_t count, first;
    if ((ps & 7u) == 0) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(ps));
        count = v.x;
        first = v.y;
    } else {
        count = __ldg(reinterpret_cast<const unsigned int*>(ps));
        first = __ldg(reinterpret_cast<const unsigned int*>(ps + 4));
    }
    const uint32_t num_matrices = __ldg(reinterpret_cast<const unsigned int*>(ml));
    indirect = make_uint4(count, num_matrices, first, 0u);
    p0 = make_ulonglong2(vtx, idx);
    p1 = make_ulonglong2(ml, dd);
}

}  // namespace cadr
