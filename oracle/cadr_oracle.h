/*
 * cadr_oracle.h - CPU oracle of the drawable-processing pass.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA path is
 * compared against (tests/, __graft_entry__.smoke) and the CPU baseline that
 * bench.py times.  The product path (libcadr_cuda.so) never links or calls it.
 *
 * Tier A follows src/CadR/shaders/processDrawables.comp:77-113 of the CADR
 * reference bit for bit.  Tier B has no implementation in the reference; it
 * follows the pass specification frozen by this project, which reuses the
 * reference's own arithmetic where the reference has it:
 *   matrix product order  examples/gltfReader/main.cpp:1546 (m = parent * node)
 *                         with GLM's mat4 operator* (glm/detail/type_mat4x4.inl)
 *   sphere transform      src/CadR/BoundingSphere.h:70-86
 *   StateSet regions      src/CadR/StateSet.cpp:233-261
 * Build with -ffp-contract=off: every float operation is rounded on its own,
 * in the order written, exactly as the CUDA kernels do with __fmul_rn and
 * __fadd_rn.
 */
#ifndef CADR_ORACLE_H
#define CADR_ORACLE_H

#include <stdint.h>
#include "../include/cadr_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Tier A over a host image of device memory: the bytes of
 * [image_base, image_base + image_size) as the GPU would see them.
 * Returns 0, or -1 when a lookup leaves the image (the GPU would read
 * unrelated memory there). */
int oracle_process_drawables(const uint8_t* image, uint64_t image_base, uint64_t image_size,
                             uint32_t handle_level, uint64_t handle_table_addr,
                             const cadr_drawable_gpu_data* drawables, uint64_t n,
                             cadr_draw_indirect_cmd* indirect, cadr_drawable_pointers* pointers,
                             int threads);

/* The same over several regions of device memory (e.g. the DataMemory
 * blocks of a DataStorage, downloaded to the host). */
typedef struct oracle_region {
    const uint8_t* bytes;
    uint64_t base;
    uint64_t size;
} oracle_region;
int oracle_process_drawables_regions(const oracle_region* regions, uint32_t num_regions,
                                     uint32_t handle_level, uint64_t handle_table_addr,
                                     const cadr_drawable_gpu_data* drawables, uint64_t n,
                                     cadr_draw_indirect_cmd* indirect,
                                     cadr_drawable_pointers* pointers, int threads);

/* StateSet packing of StateSet::prepareRecording / recordToCommandBuffer
 * (src/CadR/StateSet.cpp:180-268): the StateSets are visited in
 * depth-first order dfs_order[0..S-1]; each copies its drawable list (its
 * slots, in list-index order) to packed[] at the running drawableCounter,
 * which then advances by the list's length.  offsets[j] receives the
 * counter at StateSet dfs_order[j], offsets[S] the total.  Returns -1 for a
 * layout that is not a set of lists (a StateSet or list index out of range,
 * a list index used twice, dfs_order not a permutation). */
int oracle_pack_state_sets(uint32_t S, const uint32_t* dfs_order, uint64_t n, const uint32_t* state_set_of_slot,
                           const uint32_t* list_index_of_slot, const cadr_drawable_gpu_data* pool,
                           cadr_drawable_gpu_data* packed, uint32_t* offsets);

/* The vertex-pulling consumer check of cadr_check_draws, over host copies
 * of the device memory regions: same reads, same arithmetic, same flags
 * and checksums (see include/cadr_cuda.h). */
int oracle_check_draws(const oracle_region* regions, uint32_t num_regions, const cadr_draw_indirect_cmd* indirect,
                       const cadr_drawable_pointers* pointers, uint64_t n, const cadr_consumer_view* view,
                       cadr_draw_check* out, int threads);

/* GLM-order 4x4 product out = a * b (column-major float[16]). */
void oracle_mat4_mul(const float* a, const float* b, float* out);
/* BoundingSphere operator*: out = m * (cx, cy, cz, r). */
void oracle_sphere_transform(const float* m, const float* sphere, float* out);

/* world[i] = parent_world[parent[i]] * local[i]; parent == NULL means
 * world = local.  Returns -1 when a parent index is >= num_parents. */
int oracle_propagate(const float* parent_world, uint64_t num_parents, const float* local,
                     const uint32_t* parent, uint64_t n, float* world, int threads);

/* Per-drawable classification of one view: visible flag, LOD and marginal
 * flag of a world sphere. */
void oracle_classify(const float* world_sphere, const cadr_view* view, uint32_t num_lods,
                     int* visible, uint32_t* lod, int* marginal);

/* Full plain pass over a scene held in host arrays.
 *   levels: num_levels internal levels, level_local[l] (n_l*16 floats),
 *           level_parent[l] (n_l, NULL for level 0).
 *   leaf:   local (N*16), parent (N, may be NULL when num_levels == 0),
 *           sphere (N*4), geometry (N), state_set_offsets (S+1), lods (G*L).
 * Outputs (any may be NULL except cmds and counts): cmds (N), counts (S),
 * marginal (ceil(N/32) words), world (N*16), world_sphere (N*4).
 * Returns 0, or -1 on an invalid index or unsorted offsets. */
int oracle_cull(uint32_t num_levels, const uint64_t* level_size, const float* const* level_local,
                const uint32_t* const* level_parent, uint64_t n, const float* local,
                const uint32_t* parent, const float* sphere, const uint32_t* geometry,
                uint32_t num_state_sets, const uint32_t* state_set_offsets,
                uint32_t num_geometries, uint32_t num_lods, const cadr_lod* lods,
                const cadr_view* view, cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                uint32_t* marginal, float* world, float* world_sphere, int threads);

/* Cull of one view from precomputed world spheres (the batched form's
 * per-view work: identical arithmetic to the tail of oracle_cull). */
int oracle_cull_spheres(uint64_t n, const float* world_sphere, const uint32_t* geometry,
                        uint32_t num_state_sets, const uint32_t* state_set_offsets,
                        uint32_t num_geometries, uint32_t num_lods, const cadr_lod* lods,
                        const cadr_view* view, cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                        uint32_t* marginal, int threads);

/* Number of OpenMP threads available (1 when built without OpenMP). */
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
