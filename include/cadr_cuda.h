/*
 * cadr_cuda.h - C ABI of the GB300 (sm_103a) drawable-processing pass.
 *
 * Every entry point takes plain pointers and sizes.  Device buffers are raw
 * device pointers (the CUDA equivalent of a VkDeviceAddress); streams are
 * cudaStream_t values passed as `void*` (NULL = the context's own stream).
 * No C++ exception crosses this boundary: every call returns a cadr_status,
 * and cadr_last_error() gives a one-line description of the last failure on
 * the calling thread.
 *
 * Two tiers share one context:
 *   Tier A  cadr_process_drawables: the handle-resolution pass of the
 *           reference's processDrawables compute shader, bit-exact.
 *   Tier B  cadr_cull / cadr_cull_batched / cadr_server_*: hierarchy
 *           propagation, bounding-sphere frustum culling with screen-size LOD
 *           selection and deterministic per-StateSet compaction into
 *           VkDrawIndexedIndirectCommand records.
 *
 * Reference interfaces replaced (paths inside the CADR project):
 *   src/CadR/Renderer.cpp:598-720   Renderer::recordDrawableProcessing
 *   src/CadR/shaders/processDrawables.comp:68-113  push constants + main()
 *   src/CadR/StateSet.cpp:198-268   per-StateSet regions and draw counts
 *   src/CadR/Renderer.cpp:946-999   Renderer::executeCopyOperations (uploads)
 */
#ifndef CADR_CUDA_H
#define CADR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define CADR_API __declspec(dllexport)
#else
#define CADR_API __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------------------ */
/* Status codes.  They mirror the reference's exception classes
 * (src/CadR/Exceptions.h:13-40): OUT_OF_MEMORY <-> CadR::OutOfResources,
 * TIMEOUT <-> CadR::Timeout, INVALID_ARG <-> CadR::LogicError.            */
typedef enum cadr_status {
    CADR_OK = 0,
    CADR_ERR_INVALID_ARG = 1,
    CADR_ERR_OUT_OF_MEMORY = 2,
    CADR_ERR_TIMEOUT = 3,      /* a bounded device wait expired (lookback, mbarrier) */
    CADR_ERR_CUDA = 4,         /* a CUDA runtime call failed */
    CADR_ERR_DEVICE = 5,       /* a kernel reported an error through its error word */
    CADR_ERR_NOT_READY = 6,    /* polled work has not finished yet */
    CADR_ERR_REJECTED = 7      /* serving admission refused the request */
} cadr_status;

/* Device error word bits (read back by the host after a pass). */
#define CADR_DEVERR_LOOKBACK_TIMEOUT 0x1u
#define CADR_DEVERR_MBARRIER_TIMEOUT 0x2u
#define CADR_DEVERR_BAD_INDEX 0x4u
/* Set only by the bounds-checked build of this library (its sources
 * compiled with CADR_BOUNDS_CHECK defined): an index derived inside a
 * kernel (a command slot outside its StateSet region, a plane word past
 * its plane, a work item outside its job) left its range, and the access
 * it guarded was skipped. */
#define CADR_DEVERR_BOUNDS 0x8u

typedef void* cadr_stream; /* cudaStream_t */
typedef struct cadr_context cadr_context;
typedef struct cadr_scene cadr_scene;
typedef struct cadr_server cadr_server;

/* Output record layouts.  They are the Vulkan structs of the same name
 * (vulkan_core.h), restated so callers need no Vulkan headers. */
typedef struct cadr_draw_indirect_cmd { /* VkDrawIndirectCommand, 16 B */
    uint32_t vertex_count;
    uint32_t instance_count;
    uint32_t first_vertex;
    uint32_t first_instance;
} cadr_draw_indirect_cmd;

typedef struct cadr_draw_indexed_cmd { /* VkDrawIndexedIndirectCommand, 20 B */
    uint32_t index_count;
    uint32_t instance_count;
    uint32_t first_index;
    int32_t vertex_offset;
    uint32_t first_instance;
} cadr_draw_indexed_cmd;

/* Tier A input record: CadR::DrawableGpuData, 48 B (src/CadR/Drawable.h:32-43). */
typedef struct cadr_drawable_gpu_data {
    uint64_t vertex_data_handle;
    uint64_t index_data_handle;
    uint64_t matrix_list_handle;
    uint64_t drawable_data_handle;
    uint64_t primitive_set_handle;
    uint32_t primitive_set_offset;
    uint32_t padding;
} cadr_drawable_gpu_data;

/* Tier A second output: the 32 B DrawablePointers record
 * (src/CadR/shaders/processDrawables.comp:52-59, Renderer.h:201). */
typedef struct cadr_drawable_pointers {
    uint64_t vertex_data_ptr;
    uint64_t index_data_ptr;
    uint64_t matrix_list_ptr;
    uint64_t drawable_data_ptr;
} cadr_drawable_pointers;

/* One LOD of a geometry: the PrimitiveSet {indexCount, startIndex}
 * (src/CadR/PrimitiveSet.h:12-15) plus the vertex offset of an indexed draw.
 * Padded to 16 B so one vector load fetches it. */
typedef struct cadr_lod {
    uint32_t index_count;
    uint32_t first_index;
    int32_t vertex_offset;
    uint32_t reserved;
} cadr_lod;

/* One view (camera or shadow cascade), precomputed on the host.
 *   planes[p] = (nx, ny, nz, d): a sphere (c, r) is outside plane p when
 *               ((nx*cx + ny*cy) + nz*cz) + d < -r.
 *   view_z    = row 2 of the view matrix: z_view = ((vz0*cx + vz1*cy) + vz2*cz) + vz3.
 *   LOD:      zc = perspective ? max(-z_view, near_z) : 1;  s = r * lod_scale;
 *             lod = first k < num_lods-1 with s >= lod_threshold[k] * zc,
 *                   else num_lods-1.                                      */
typedef struct cadr_view {
    float planes[6][4];
    float view_z[4];
    float lod_threshold[4];
    float lod_scale;
    float near_z;
    uint32_t perspective;
    uint32_t reserved;
} cadr_view; /* 144 B */

#define CADR_MAX_LEVELS 16

/* Shape of a Tier B scene: internal hierarchy levels 0..num_levels-1 followed
 * by the leaf level, which holds one world matrix per drawable.  Drawables
 * are stored grouped by StateSet, StateSet s owning the contiguous range
 * [state_set_offsets[s], state_set_offsets[s+1]) (src/CadR/StateSet.h:47,
 * StateSet.cpp:233-261). */
typedef struct cadr_scene_desc {
    uint32_t num_levels;                 /* internal levels, 0..CADR_MAX_LEVELS */
    uint32_t num_state_sets;             /* >= 1 */
    uint64_t level_size[CADR_MAX_LEVELS];
    uint64_t num_drawables;              /* < 2^32 */
    uint32_t num_geometries;             /* >= 1 */
    uint32_t num_lods;                   /* 1..4 */
} cadr_scene_desc;

/* Device-resident buffers of a scene, for callers that fill or read them in
 * place (all pointers are device pointers owned by the scene). */
typedef struct cadr_scene_buffers {
    float* level_local[CADR_MAX_LEVELS];    /* n*16 floats, column-major mat4 */
    uint32_t* level_parent[CADR_MAX_LEVELS];/* n (level 0: NULL) */
    float* level_world[CADR_MAX_LEVELS];    /* n*16 floats (level 0 aliases level_local[0]) */
    float* local;                           /* N*16 */
    uint32_t* parent;                       /* N (NULL when num_levels == 0) */
    float* sphere;                          /* N*4 local bounding spheres (cx,cy,cz,r) */
    uint32_t* geometry;                     /* N geometry index per drawable */
    uint32_t* state_set_offsets;            /* S+1 */
    cadr_lod* lods;                         /* G*num_lods */
    float* world;                           /* N*16 world matrices (written by passes) */
    float* world_sphere;                    /* N*4 world bounding spheres (written by passes) */
} cadr_scene_buffers;

/* ------------------------------------------------------------------------ */
/* Errors and context. */
CADR_API const char* cadr_status_string(cadr_status s);
CADR_API const char* cadr_last_error(void);
CADR_API int cadr_abi_version(void);
/* How this library was built: CADR_BUILD_BOUNDS_CHECK when its kernels
 * check the indices they derive (the test build; see CADR_DEVERR_BOUNDS),
 * 0 for the product build. */
#define CADR_BUILD_BOUNDS_CHECK 0x1u
CADR_API uint32_t cadr_build_flags(void);

/* Creates the per-device context: streams (compute + upload), pinned staging
 * ring and lookback scratch.  Replaces the Vulkan device/queue the reference
 * Renderer is constructed with (src/CadR/Renderer.h:124-128).  It sets the
 * process's L2 fetch granularity hint on the device to 32 bytes (the pass's
 * scattered reads are 4-16 bytes wide) and gives the previous value back in
 * cadr_context_destroy. */
CADR_API cadr_status cadr_context_create(int device, cadr_context** out);
CADR_API cadr_status cadr_context_destroy(cadr_context* ctx);
CADR_API cadr_stream cadr_context_stream(cadr_context* ctx);
CADR_API cadr_stream cadr_context_upload_stream(cadr_context* ctx);
/* Upper bound of every bounded device spin, in nanoseconds (default 1e9). */
CADR_API cadr_status cadr_context_set_spin_limit_ns(cadr_context* ctx, uint64_t ns);
CADR_API cadr_status cadr_context_synchronize(cadr_context* ctx);
/* Number of kernels this library launched through ctx since creation. */
CADR_API uint64_t cadr_context_launch_count(cadr_context* ctx);
/* Measurement aid (no reference counterpart): the HBM bandwidth, in GB/s,
 * of a kernel that moves the plain pass's leaf-stream traffic for
 * `num_drawables` drawables (64 B local + 16 B sphere + 4 B parent index
 * read, 64 B world matrix written per drawable, the stream kernel's access
 * pattern) without its arithmetic, timed over `reps` launches on the
 * context stream.  Allocates and frees 148 B per drawable. */
CADR_API cadr_status cadr_measure_stream_mix(cadr_context* ctx, uint64_t num_drawables, uint32_t reps,
                                             double* gbytes_per_s);

/* Device memory helpers (stream-ordered pool of the context's device). */
CADR_API cadr_status cadr_device_alloc(cadr_context* ctx, size_t bytes, void** out);
CADR_API cadr_status cadr_device_free(cadr_context* ctx, void* ptr);
CADR_API cadr_status cadr_host_alloc_pinned(size_t bytes, void** out);
CADR_API cadr_status cadr_host_free_pinned(void* ptr);
/* Stream-ordered copies.  Host sources that are not pinned are staged
 * through the context's pinned ring on the upload stream, which then hands
 * over to `stream` with an event (replaces DataStorage::recordUploads +
 * Renderer::executeCopyOperations, src/CadR/DataStorage.cpp:230-281,
 * Renderer.cpp:946-999, without the 1.5 s fence wait). */
CADR_API cadr_status cadr_upload(cadr_context* ctx, void* dst_device, const void* src_host,
                                 size_t bytes, cadr_stream stream);
CADR_API cadr_status cadr_download(cadr_context* ctx, void* dst_host, const void* src_device,
                                   size_t bytes, cadr_stream stream);
/* Reads the valid commands of a plain pass back to host memory: for every
 * StateSet s, the host_counts[s] records at host_offsets[s] of device_cmds
 * go to the same index of host_cmds (host_counts: the pass's counts, read
 * back first; host_offsets: the S+1 region offsets).  Regions whose valid
 * parts touch are copied together; *bytes (optional) receives the bytes
 * copied.  Stream-ordered on `stream`; host_cmds should be pinned.  No
 * reference counterpart: the reference's draws never leave the device; this
 * serves a caller that processes the culled draw list on the host. */
CADR_API cadr_status cadr_download_commands(cadr_context* ctx, cadr_draw_indexed_cmd* host_cmds,
                                            const cadr_draw_indexed_cmd* device_cmds, const uint32_t* host_counts,
                                            const uint32_t* host_offsets, uint32_t num_state_sets, uint64_t* bytes,
                                            cadr_stream stream);
CADR_API cadr_status cadr_stream_synchronize(cadr_stream stream);

/* ------------------------------------------------------------------------ */
/* Tier A.  Replaces Renderer::recordDrawableProcessing
 * (src/CadR/Renderer.cpp:598-720) and processDrawables.comp:92-113.
 * For every i < num_drawables (records already packed in StateSet
 * depth-first order, StateSet.cpp:198-262):
 *   ps = lookup(d.primitive_set_handle) + d.primitive_set_offset
 *   ml = lookup(d.matrix_list_handle)
 *   indirect[i] = {ps->count, ml->numMatrices, ps->first, 0}
 *   pointers[i] = {lookup(vertex), lookup(index), ml, lookup(drawableData)}
 * with lookup() the 1/2/3-level handle table walk of
 * processDrawables.comp:77-89 (handle_level 1..3).  Handles must be valid,
 * exactly as in the reference. */
CADR_API cadr_status cadr_process_drawables(cadr_context* ctx, uint32_t handle_level,
                                            const void* handle_table,
                                            const cadr_drawable_gpu_data* drawables,
                                            uint64_t num_drawables,
                                            cadr_draw_indirect_cmd* indirect,
                                            cadr_drawable_pointers* pointers,
                                            cadr_stream stream);

/* ------------------------------------------------------------------------ */
/* Device-resident StateSet packing of the Tier A records.  Replaces the
 * per-frame host packing of StateSet::prepareRecording and
 * StateSet::recordToCommandBuffer (src/CadR/StateSet.cpp:180-268), which
 * copies every StateSet's DrawableGpuData list, in list order and in
 * depth-first StateSet order, into the staging buffer at drawableCounter,
 * and the upload of that buffer (Renderer.cpp:635-644).  The records stay
 * in a device pool indexed by slot.  A layout gives every slot its
 * StateSet and its index in that StateSet's list, and the StateSets in
 * depth-first order; the device derives the regions and the packed
 * position of every slot.  cadr_pack_repack builds the packed array that
 * cadr_process_drawables reads; a frame whose records changed patches only
 * those rows (cadr_pack_patch) in the pool and the packed array.  Every
 * call is ordered on `stream`. */
typedef struct cadr_pack cadr_pack;
CADR_API cadr_status cadr_pack_create(cadr_context* ctx, uint32_t capacity, cadr_pack** out);
CADR_API cadr_status cadr_pack_destroy(cadr_pack* pack);
/* dfs_order[j]: the StateSet drawn j-th (a permutation of 0..num_state_sets-1);
 * state_set_of_slot[k] and list_index_of_slot[k] for the slots
 * 0..num_slots-1, the list indices of each StateSet being 0..n-1 once each.
 * A layout that breaks these rules sets CADR_DEVERR_BAD_INDEX
 * (cadr_context_check_device_error). */
CADR_API cadr_status cadr_pack_set_layout(cadr_pack* pack, uint32_t num_slots, uint32_t num_state_sets,
                                          const uint32_t* dfs_order, const uint32_t* state_set_of_slot,
                                          const uint32_t* list_index_of_slot, cadr_stream stream);
/* Records of the slots [first, first + count) from host memory, into the
 * pool; the packed array follows at the next cadr_pack_repack. */
CADR_API cadr_status cadr_pack_upload(cadr_pack* pack, const cadr_drawable_gpu_data* records, uint32_t first,
                                      uint32_t count, cadr_stream stream);
/* packed[p] = pool[slot at packed position p] for the whole layout. */
CADR_API cadr_status cadr_pack_repack(cadr_pack* pack, cadr_stream stream);
/* records[k] replaces slot slots[k], in the pool and in the packed array. */
CADR_API cadr_status cadr_pack_patch(cadr_pack* pack, const uint32_t* slots, const cadr_drawable_gpu_data* records,
                                     uint32_t count, cadr_stream stream);
/* cadr_process_drawables over the packed records [0, num_draw_records),
 * read from the pool instead of the packed array: each slot's record is
 * resolved in slot order and its indirect command and DrawablePointers are
 * written at its packed position.  The output equals cadr_process_drawables
 * on the packed array (after a repack) for those positions; no repack is
 * needed.  Slots whose packed position is num_draw_records or more are not
 * read, so they may hold any bytes (free slots).  With slots handed out in
 * drawable creation order, the handle-table reads of neighbouring slots
 * are neighbours too. */
CADR_API cadr_status cadr_pack_process_drawables(cadr_pack* pack, uint32_t handle_level, const void* handle_table,
                                                 uint32_t num_draw_records, cadr_draw_indirect_cmd* indirect,
                                                 cadr_drawable_pointers* pointers, cadr_stream stream);
/* Device pointers: the packed records (num_slots of them) and the region
 * offsets (num_state_sets + 1): StateSet dfs_order[j] occupies packed
 * records [offsets[j], offsets[j+1]), which is the reference's
 * drawableCounter at that StateSet; its draw is
 * cmdDrawIndirect(offset = offsets[j] * 16, count = offsets[j+1] - offsets[j])
 * over cadr_process_drawables' output. */
CADR_API cadr_status cadr_pack_buffers(cadr_pack* pack, const cadr_drawable_gpu_data** packed,
                                       const uint32_t** region_offsets, uint32_t* num_slots);

/* ------------------------------------------------------------------------ */
/* Vertex-pulling consumer check of the Tier A draws.  Replays, in CUDA, the
 * reads of the vertex shader that consumes them
 * (examples/RenderingPerformance/shader.vert:100-120): for draw i of
 * cmdDrawIndirect, with dp = pointers[i] and cmd = indirect[i], for every
 * instance m in [firstInstance, firstInstance + instanceCount) and vertex
 * v = firstVertex + k, k < vertexCount:
 *   index    = ((const uint32_t*)dp.index_data)[v]
 *   position = ((const float[3]*)dp.vertex_data)[index]
 *   eye      = (view * matrixList(dp.matrix_list).matrices[m]) * (position, 1)
 *   gl_Position = (p11 ex + p31 ez + p41 ew, p22 ey + p32 ez + p42 ew,
 *                  p33 ez + p43 ew, p34 ez + p44 ew),  eye3 = eye.xyz / eye.w
 * (GLM operation order, every operation rounded once).  Every address is
 * checked against `regions` (the device memory the draws may address) and
 * against its alignment before it is read: a read that fails is skipped
 * and flagged, so a bad draw buffer cannot fault the device.  Per draw:
 * the (vertex, instance) pairs pulled, the flags, and the checksum: the sum
 * modulo 2^64 over those pairs of
 *   mix(X | Y << 32) ^ mix((Z | W << 32) ^ K) ^ mix((EX | EY << 32) ^ 2K)
 *   ^ mix((EZ | index << 32) ^ 3K)
 * with X..W the bits of gl_Position, EX..EZ those of eye3, K =
 * 0x9E3779B97F4A7C15 and mix the SplitMix64 finaliser (order-independent,
 * so any thread layout gives the same sum). */
typedef struct cadr_memory_region {
    uint64_t base;
    uint64_t size;
} cadr_memory_region;
#define CADR_MAX_MEMORY_REGIONS 8u
typedef struct cadr_consumer_view {
    float view[16];                       /* SceneData.viewMatrix, column-major */
    float p11, p22, p33, p43;             /* SceneData projection members */
    float p31, p32, p34, p41, p42, p44;   /* specialization constants */
    uint32_t reserved[2];
} cadr_consumer_view;
typedef struct cadr_draw_check {
    uint64_t checksum;
    uint32_t pulled;   /* (vertex, instance) pairs read and transformed */
    uint32_t flags;    /* CADR_DRAW_* */
} cadr_draw_check;
#define CADR_DRAW_BAD_INDEX_READ 0x1u     /* an index read outside the regions or misaligned */
#define CADR_DRAW_BAD_VERTEX_READ 0x2u    /* a position read outside the regions or misaligned */
#define CADR_DRAW_BAD_MATRIX_LIST 0x4u    /* header or a matrix outside the regions, or not 64-byte aligned */
#define CADR_DRAW_BAD_INSTANCE 0x8u       /* an instance index >= numMatrices */
#define CADR_DRAW_BAD_DRAWABLE_DATA 0x10u /* non-null drawable data outside the regions or misaligned */
CADR_API cadr_status cadr_check_draws(cadr_context* ctx, const cadr_draw_indirect_cmd* indirect,
                                      const cadr_drawable_pointers* pointers, uint64_t num_draws,
                                      const cadr_memory_region* regions, uint32_t num_regions,
                                      const cadr_consumer_view* view, cadr_draw_check* out,
                                      cadr_stream stream);

/* ------------------------------------------------------------------------ */
/* Tier B scenes. */
CADR_API cadr_status cadr_scene_create(cadr_context* ctx, const cadr_scene_desc* desc,
                                       cadr_scene** out);
CADR_API cadr_status cadr_scene_destroy(cadr_scene* scene);
CADR_API cadr_status cadr_scene_get_buffers(cadr_scene* scene, cadr_scene_buffers* out);
/* Host uploads of scene inputs (rows [first, first+count) of one array).
 * `parent` may be NULL to leave the parent array untouched.  Uploads run
 * on the context's upload stream in call order.  An upload waits there for
 * the passes issued before it that read the scene (cadr_cull,
 * cadr_cull_static_scratch, cadr_scene_propagate, cadr_cull_batched), and
 * the passes issued after it wait for the upload, so a frame loop may
 * upload the next frame's inputs without synchronising.  Scenes served by a
 * cadr_server are read on the server's own streams: drain the server
 * before uploading into them. */
CADR_API cadr_status cadr_scene_upload_level(cadr_scene* scene, uint32_t level,
                                             const float* local, const uint32_t* parent,
                                             uint64_t first, uint64_t count);
CADR_API cadr_status cadr_scene_upload_drawables(cadr_scene* scene, const float* local,
                                                 const uint32_t* parent, const float* sphere,
                                                 const uint32_t* geometry, uint64_t first,
                                                 uint64_t count);
CADR_API cadr_status cadr_scene_upload_state_sets(cadr_scene* scene, const uint32_t* offsets);
CADR_API cadr_status cadr_scene_upload_lods(cadr_scene* scene, const cadr_lod* lods);
/* Re-validates the scene after in-place device writes (parents monotone?
 * offsets sorted?) and orders uploads before the next pass. */
CADR_API cadr_status cadr_scene_commit(cadr_scene* scene);

/* Propagates the internal hierarchy levels (level l world =
 * level l-1 world[parent] * local, level by level) and, when
 * write_world_spheres is set, the leaf world matrices and world spheres that
 * cadr_cull_batched consumes. */
CADR_API cadr_status cadr_scene_propagate(cadr_scene* scene, int write_world_spheres,
                                          cadr_stream stream);

/* Plain pass: propagation of every level, then one fused leaf kernel that
 * computes world matrices, transforms the bounding spheres
 * (src/CadR/BoundingSphere.h:70-86), culls them against the 6 planes,
 * selects the LOD and compacts visible drawables of StateSet s into
 * cmds[offsets[s] .. offsets[s]+counts[s]) in ascending drawable order.
 * cmds: N records; counts: S words; marginal: optional ceil(N/32) words, bit i
 * set when the surface of drawable i's world sphere lies within 1e-5 of a
 * plane, |dist + r| <= 1e-5 in world units (reported, not special-cased). */
CADR_API cadr_status cadr_cull(cadr_scene* scene, const cadr_view* view,
                               cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                               uint32_t* marginal, cadr_stream stream);

/* The plain pass without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory while they run: a renderer whose device memory is owned and
 * budgeted by the host application, or a frame loop that cannot afford the
 * device-wide synchronisation of cudaMalloc/cudaFree, which cadr_cull may
 * perform when a scene needs more scratch than it holds.  Same
 * kernels and bit-identical results as cadr_cull; the caller still passes
 * the outputs.  The scratch is a static device array of 12 MiB + 128 KiB
 * (held by every GPU that loads the library until exit), which limits scenes
 * to 33,554,432 drawables; larger ones are rejected with
 * CADR_ERR_INVALID_ARG, as are scenes not committed yet.  The first call on
 * a device looks up the array's device address (set-up): make that first
 * call before any stream capture.  Every call shares the one array, so
 * calls whose work overlaps on the GPU race.  Each call is ordered after the
 * context's previous plain pass (cadr_cull or this entry point, on any
 * stream), as cadr_cull calls are; calls through different contexts on one
 * device, and cadr_scene_propagate on the same scene from another stream,
 * must be ordered by the caller. */
CADR_API cadr_status cadr_cull_static_scratch(cadr_scene* scene, const cadr_view* view,
                                              cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                                              uint32_t* marginal, cadr_stream stream);

/* Sharded plain pass: one device's part of a pass whose drawables are split
 * over several devices, as contiguous ranges [lo, hi) of the StateSet-grouped
 * drawables.  The reference runs the pass on one queue (src/CadR/
 * Renderer.cpp:108); this is the split of the same pass, so that the merged
 * output is, word for word, that of cadr_cull on the whole scene.  `scene`
 * holds the shard: its drawables, the internal levels (replicated), and the
 * StateSet offsets clipped to the range and taken relative to lo.
 *
 * Phase 1, cadr_cull_shard_count: propagation, culling and LOD of the
 * shard; counts[s] (S words, device) receives its visible drawables in
 * StateSet region s, marginal (optional) its marginal bits.  The ranks then
 * exchange their counts (an all-gather of S words: the pass's one exchange
 * step).  Phase 2, cadr_cull_shard_write: rank r writes its k-th visible
 * drawable of region s at cmds[dst_base[s] + k] with
 *   dst_base[s] = offsets[s] + sum_{q < r} count[q][s]
 * (offsets of the whole scene; dst_base is S words of device memory) and
 * firstInstance = its index in the shard + first_instance (= lo).  `cmds` is
 * the merged buffer of cmd_capacity records; a slot outside it is flagged
 * CADR_DEVERR_BAD_INDEX and not written.  Counts of the merged pass are the
 * sums over ranks.  The write must follow the count of the same scene on
 * the same context, with no upload into the scene between them; a second
 * count replaces a pending one. */
CADR_API cadr_status cadr_cull_shard_count(cadr_scene* scene, const cadr_view* view, uint32_t* counts,
                                           uint32_t* marginal, cadr_stream stream);
CADR_API cadr_status cadr_cull_shard_write(cadr_scene* scene, const uint32_t* dst_base,
                                           uint32_t first_instance, cadr_draw_indexed_cmd* cmds,
                                           uint64_t cmd_capacity, cadr_stream stream);

/* Batched form: many (scene, view) pairs culled by one persistent launch over
 * (view, tile) work items, replayed from a captured CUDA graph when the
 * same batch shape repeats.  Scenes must have been propagated with
 * write_world_spheres = 1. */
typedef struct cadr_batch_view {
    cadr_scene* scene;
    cadr_view view;
    cadr_draw_indexed_cmd* cmds;  /* device, scene N records */
    uint32_t* counts;             /* device, scene S words */
    uint32_t* marginal;           /* device or NULL */
} cadr_batch_view;

/* form 0 (CADR_BATCHED_PERSISTENT): one persistent launch over (view, tile)
 * items of block_threads * items_per_thread drawables, compacting with a
 * decoupled lookback between tiles; grid = ctas_per_sm * SMs.
 * form 1 (CADR_BATCHED_THREE_LAUNCH): three launches (classify, a per-view
 * scan of the tiles' counts, write) over tiles of 2,048 drawables with no
 * waits between CTAs, as the plain pass; it takes block_threads 256 and
 * items_per_thread 8.  Both give identical outputs. */
#define CADR_BATCHED_PERSISTENT 0u
#define CADR_BATCHED_THREE_LAUNCH 1u
typedef struct cadr_tuning {
    uint32_t block_threads;       /* 128, 256, 512 */
    uint32_t items_per_thread;    /* 4, 8, 16 */
    uint32_t ctas_per_sm;         /* persistent grid = ctas_per_sm * SMs, 1..16 */
    uint32_t form;                /* CADR_BATCHED_* */
} cadr_tuning;

CADR_API cadr_status cadr_cull_batched(cadr_context* ctx, const cadr_batch_view* views,
                                       uint32_t num_views, const cadr_tuning* tuning,
                                       int use_graph, cadr_stream stream);
/* Autotuner: times every supported tuning on this batch (CUDA events, median
 * of `reps` runs) and keeps the fastest as the context's default.  With a
 * tuning cache set (cadr_context_set_tuning_cache), the pick is stored under
 * a key of the batch's shape (per view: the scene's drawables, StateSets and
 * LODs), the GPU (name, SMs, compute capability) and the driver version, and
 * a later batch with the same key takes it from the cache without timing.
 * The reference has no tuner: its dispatch shape is fixed (Renderer.cpp:684-692). */
CADR_API cadr_status cadr_autotune_batched(cadr_context* ctx, const cadr_batch_view* views,
                                           uint32_t num_views, uint32_t reps, cadr_tuning* best,
                                           float* best_ms);
/* The cache file of the context's autotuner (NULL or "" = no cache). */
CADR_API cadr_status cadr_context_set_tuning_cache(cadr_context* ctx, const char* path);
/* The search and the cache without a GPU: cadr_autotune_with times every
 * supported tuning with time_fn (which returns CADR_OK and the time of one
 * tuning in *ms) and keeps the fastest; with cache_path set it first looks
 * `key` up there (then *from_cache = 1 and time_fn is not called) and stores
 * its pick afterwards.  cadr_tuning_cache_lookup returns CADR_ERR_NOT_READY
 * when the key is absent.  Keys may not hold quotes, backslashes or line
 * breaks. */
typedef cadr_status (*cadr_time_tuning_fn)(const cadr_tuning* tuning, void* user, float* ms);
CADR_API cadr_status cadr_autotune_with(const char* cache_path, const char* key, cadr_time_tuning_fn time_fn,
                                        void* user, cadr_tuning* best, float* best_ms, int* from_cache);
CADR_API cadr_status cadr_tuning_cache_lookup(const char* path, const char* key, cadr_tuning* out, float* ms);
CADR_API cadr_status cadr_tuning_cache_store(const char* path, const char* key, const cadr_tuning* tuning,
                                             float ms);
CADR_API cadr_status cadr_get_tuning(cadr_context* ctx, cadr_tuning* out);
CADR_API cadr_status cadr_set_tuning(cadr_context* ctx, const cadr_tuning* tuning);

/* Frame timing, the CUDA counterpart of CadR::FrameInfo's GPU timestamps
 * (src/CadR/FrameInfo.h:15-31, collected in Renderer.cpp:600-702): while
 * collection is on, every plain pass records events before propagation,
 * after each internal level, between propagation and the leaf stage, after
 * the stream kernel and after the leaf stage, into a ring of 256 frames.
 * get_frame_infos waits for and returns the frames finished since the
 * previous call.  A pass with frame timing launches its kernels one after
 * the other (no programmatic overlap across the recorded events), so its
 * times are each kernel's own. */
typedef struct cadr_frame_info {
    uint64_t frame;
    float propagate_ms;     /* internal hierarchy levels */
    float leaf_ms;          /* leaf stage: stream, tile scan and write kernels */
    float total_ms;
    float stream_ms;        /* the leaf stream kernel alone (part of leaf_ms) */
    uint32_t num_levels;    /* internal levels of the scene */
    float level_ms[CADR_MAX_LEVELS]; /* level l's propagation (level 0 has none: 0) */
} cadr_frame_info;
CADR_API cadr_status cadr_context_set_collect_frame_info(cadr_context* ctx, int on);
CADR_API cadr_status cadr_context_get_frame_infos(cadr_context* ctx, cadr_frame_info* out,
                                                  uint32_t max_frames, uint32_t* num_frames);

/* GPU timestamps of the C++ facade's frames, for CadR::FrameInfo's four
 * GPU fields (src/CadR/FrameInfo.h:26-29: begin of execution, after the
 * transfers, after drawable processing, end of execution; written in
 * Renderer.cpp:600-702).  record_timestamp records timestamp `index`
 * (0..3) of frame `frame` on `stream` (null: the context's stream); the last
 * 4 frames are kept.  read_timestamps waits for the frame's four timestamps
 * and returns them in out_ns[4] as nanoseconds after timestamp 0
 * (out_ns[0] = 0); CADR_ERR_INVALID_ARG when the frame has not recorded all
 * four or was overwritten. */
CADR_API cadr_status cadr_context_record_timestamp(cadr_context* ctx, uint64_t frame, uint32_t index,
                                                  cadr_stream stream);
CADR_API cadr_status cadr_context_read_timestamps(cadr_context* ctx, uint64_t frame, uint64_t* out_ns);

/* Host-side check of the last pass's device error word (0 = no error). */
CADR_API cadr_status cadr_context_check_device_error(cadr_context* ctx, uint32_t* error_bits);

/* Fault injection for the bounded-wait tests: while set, the first tile of
 * every view of a batched pass (cadr_cull_batched) never publishes its
 * lookback status, so its successors' waits run into the spin limit and
 * cadr_context_check_device_error returns CADR_ERR_TIMEOUT.  The pass still
 * ends; the context stays usable.  (The plain pass has no waits.) */
#define CADR_FAULT_NONE 0u
#define CADR_FAULT_SKIP_FIRST_TILE_PUBLISH 1u
/* Host side, for the serving tests: while set, every batch a server on this
 * context admits fails before anything is launched, as a failed launch
 * would; its requests finish with CADR_ERR_CUDA and give their output
 * memory back.  No GPU work is involved. */
#define CADR_FAULT_SERVER_LAUNCH 2u
CADR_API cadr_status cadr_debug_set_fault(cadr_context* ctx, uint32_t fault);

/* ------------------------------------------------------------------------ */
/* Serving form: a request loop over resident scenes with continuous
 * batching.  Requests are admitted as output memory and slots free up;
 * admitted requests are batched within a window and culled by the batched
 * kernel on one of several streams, so batches overlap on the device. */
typedef struct cadr_server_config {
    uint32_t max_inflight_batches; /* streams in rotation, >= 1 */
    uint32_t max_batch_views;      /* views per batch */
    uint64_t window_ns;            /* batching window, e.g. 200000: the longest a request waits for
                                      others; none while no batch is in flight or once the pending
                                      work fills the device */
    uint64_t memory_budget_bytes;  /* output memory the server may hold (0 = from free memory) */
    uint64_t reserve_bytes;        /* free device memory left untouched */
} cadr_server_config;

typedef struct cadr_request_result {
    uint64_t request_id;
    cadr_status status;
    uint32_t num_views;
    uint64_t submit_ns;            /* host monotonic clock */
    uint64_t complete_ns;
    const cadr_draw_indexed_cmd* cmds[4]; /* device pointers, valid until released */
    const uint32_t* counts[4];
} cadr_request_result;

CADR_API cadr_status cadr_server_create(cadr_context* ctx, const cadr_server_config* cfg,
                                        cadr_server** out);
CADR_API cadr_status cadr_server_destroy(cadr_server* srv);
CADR_API cadr_status cadr_server_submit(cadr_server* srv, cadr_scene* scene,
                                        const cadr_view* views, uint32_t num_views,
                                        uint64_t* request_id);
/* Returns up to max_results finished requests (CADR_OK with *num_results 0
 * when none finished). */
CADR_API cadr_status cadr_server_poll(cadr_server* srv, cadr_request_result* results,
                                      uint32_t max_results, uint32_t* num_results);
CADR_API cadr_status cadr_server_release(cadr_server* srv, uint64_t request_id);
CADR_API cadr_status cadr_server_drain(cadr_server* srv);

/* ------------------------------------------------------------------------ */
/* Output buffers shared with a Vulkan renderer.  The reference shares
 * memory between APIs by allocating it exportable and handing an opaque
 * file descriptor to the importer (examples/OpenGLInteroperability/
 * main.cpp:1488-1490, 1538-1550, 1616-1619).  A shared buffer is device
 * memory made for POSIX-FD export and mapped into the context; the pass
 * writes its commands, counts, indirect records or pointers straight into
 * it, and a Vulkan device imports the descriptor with
 * VkImportMemoryFdInfoKHR (VK_EXTERNAL_MEMORY_HANDLE_TYPE_OPAQUE_FD_BIT,
 * allocationSize = cadr_shared_buffer_size) and draws from it. */
typedef struct cadr_shared_buffer cadr_shared_buffer;
/* `bytes` is rounded up to the allocation granularity. */
CADR_API cadr_status cadr_shared_buffer_create(cadr_context* ctx, size_t bytes, cadr_shared_buffer** out);
CADR_API void* cadr_shared_buffer_device_ptr(cadr_shared_buffer* buf);
CADR_API size_t cadr_shared_buffer_size(cadr_shared_buffer* buf);
/* A new descriptor for every call; the importer owns it (Vulkan takes
 * ownership on a successful import, otherwise the caller closes it). */
CADR_API cadr_status cadr_shared_buffer_export_fd(cadr_shared_buffer* buf, int* fd);
/* Maps an exported descriptor of `bytes` (cadr_shared_buffer_size of the
 * exporter) into ctx: the same memory at a second address.  The caller
 * keeps the descriptor and closes it. */
CADR_API cadr_status cadr_shared_buffer_import_fd(cadr_context* ctx, int fd, size_t bytes,
                                                  cadr_shared_buffer** out);
/* Waits for the device, then unmaps and releases (the memory itself lives
 * on while another mapping or an importer holds it). */
CADR_API cadr_status cadr_shared_buffer_destroy(cadr_shared_buffer* buf);

#ifdef __cplusplus
}
#endif

#endif /* CADR_CUDA_H */
