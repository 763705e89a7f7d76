/* ref_shader_shim.h - compiles the CADR reference's processDrawables
 * compute shader (src/CadR/shaders/processDrawables.comp), unchanged but for
 * its #version and #extension lines, as C++ on the host, so that Tier A's
 * oracle can be checked against the reference's own shader code.
 *
 * TEST INFRASTRUCTURE ONLY.  Force-included (-include) by `make -C oracle
 * ref` into each of three compilations of the shader (one per handle-table
 * depth); the result goes to oracle/_ref/ and is driven by
 * ref_shader_harness.cpp.
 *
 * GLSL constructs and their C++ stand-ins:
 *   layout(...), restrict, readonly, writeonly, `in`  no meaning on the host
 *   `buffer X { ... };`                  struct X { ... };
 *   `uniform pushConstants { ... };`     struct pushConstants { ... } (unused);
 *                                        its members are the globals below
 *   X(address)  (buffer_reference cast)  pointer to the block at the address
 *   the shader's reference variables     names bound to those pointers
 *   uint64_t(reference)                  the block's address
 *   uint, mat4, gl_WorkGroupID           uint32_t, 16 floats, a global
 * Every memory access of the shader thus reads or writes host memory at the
 * addresses its handle tables hold, with the shader's own integer widths
 * and truncations. */
#ifndef CADR_REF_SHADER_SHIM_H
#define CADR_REF_SHADER_SHIM_H

#include <cstdint>

typedef uint32_t uint;
struct mat4 {
    float m[16];
};
struct cadr_uvec3 {
    uint32_t x, y, z;
};
extern cadr_uvec3 gl_WorkGroupID;

struct HandleTableRef;
extern HandleTableRef* cadr_handle_table;
extern uint64_t cadr_drawable_list_ptr, cadr_indirect_data_ptr, cadr_drawable_pointers_ptr;

template <class T>
inline uint64_t cadr_u64(T& block)
{
    return (uint64_t)reinterpret_cast<uintptr_t>(&block);
}
inline uint64_t cadr_u64(uint64_t v) { return v; }

#define layout(...)
#define restrict
#define readonly
#define writeonly
#define in
#define buffer struct
#define uniform struct

#define DrawableGpuDataRef(a) reinterpret_cast<DrawableGpuDataRef*>(a)
#define PrimitiveSetRef(a) reinterpret_cast<PrimitiveSetRef*>(a)
#define MatrixListRef(a) reinterpret_cast<MatrixListRef*>(a)
#define IndirectDataRef(a) reinterpret_cast<IndirectDataRef*>(a)
#define DrawablePointersRef(a) reinterpret_cast<DrawablePointersRef*>(a)
#define HandleTableRef(a) reinterpret_cast<HandleTableRef*>(a)

#define d (*cadr_v_d)
#define ps (*cadr_v_ps)
#define ml (*cadr_v_ml)
#define indirectData (*cadr_v_indirect)
#define dp (*cadr_v_dp)
#define table2 (*cadr_v_table2)
#define table3 (*cadr_v_table3)

#define handleTable (*cadr_handle_table)
#define drawableListPtr cadr_drawable_list_ptr
#define indirectDataPtr cadr_indirect_data_ptr
#define drawablePointersBufferPtr cadr_drawable_pointers_ptr

#define uint64_t(x) cadr_u64(x)

#endif
