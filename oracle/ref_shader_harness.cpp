// ref_shader_harness.cpp - runs the CADR reference's processDrawables shader,
// compiled as C++ through ref_shader_shim.h, over a host memory image: one
// call of the shader's main() per drawable, with gl_WorkGroupID set as the
// reference's dispatch sets it (x = i % 32768, y = i / 32768,
// Renderer.cpp:684-692).
//
// TEST INFRASTRUCTURE ONLY (see ref_shader_shim.h).  Linked with the three
// compilations of the shader into oracle/_ref/libcadr_ref_shader.so.
#include <cstdint>

#include <sys/mman.h>

struct HandleTableRef;
struct cadr_uvec3 {
    uint32_t x, y, z;
};

cadr_uvec3 gl_WorkGroupID;
HandleTableRef* cadr_handle_table;
uint64_t cadr_drawable_list_ptr, cadr_indirect_data_ptr, cadr_drawable_pointers_ptr;

void cadr_ref_shader_main_l1();
void cadr_ref_shader_main_l2();
void cadr_ref_shader_main_l3();

// Maps `size` bytes of zeroed memory at exactly `base`, so that an image laid
// out for that address can be run at it; 0 on success, -1 when the range is
// taken or the mapping fails (never replaces an existing mapping).
extern "C" __attribute__((visibility("default"))) int cadr_ref_shader_map(uint64_t base, uint64_t size)
{
    void* want = reinterpret_cast<void*>(base);
    void* p = mmap(want, size, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_FIXED_NOREPLACE, -1, 0);
    if (p == MAP_FAILED) return -1;
    if (p != want) {
        munmap(p, size);
        return -1;
    }
    return 0;
}

extern "C" __attribute__((visibility("default"))) int cadr_ref_shader_unmap(uint64_t base, uint64_t size)
{
    return munmap(reinterpret_cast<void*>(base), size);
}

extern "C" __attribute__((visibility("default"))) int cadr_ref_shader_process(uint32_t handle_level, uint64_t root,
                                                                              uint64_t drawables, uint64_t n,
                                                                              uint64_t indirect, uint64_t pointers)
{
    if (handle_level < 1 || handle_level > 3) return -1;
    cadr_handle_table = reinterpret_cast<HandleTableRef*>(root);
    cadr_drawable_list_ptr = drawables;
    cadr_indirect_data_ptr = indirect;
    cadr_drawable_pointers_ptr = pointers;
    for (uint64_t i = 0; i < n; i++) {
        gl_WorkGroupID = cadr_uvec3{(uint32_t)(i % 32768), (uint32_t)(i / 32768), 0u};
        if (handle_level == 1)
            cadr_ref_shader_main_l1();
        else if (handle_level == 2)
            cadr_ref_shader_main_l2();
        else
            cadr_ref_shader_main_l3();
    }
    return 0;
}
