// kernels.cuh - launch interface between the C ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace cadr {

// Scratch of one running pass: lookback control block + tile states.
struct Scratch {
    LookbackCtl* ctl = nullptr;
    uint64_t* tile_state = nullptr;
    uint64_t capacity = 0;      // tile states available
    uint64_t launches = 0;      // passes run since the last full reset
    uint32_t* planes = nullptr; // plain pass: visibility and LOD bit-planes
    uint64_t plane_words = 0;   // words available in `planes`
};

struct LeafArgs {
    const float4* local;          // N * 4 columns
    const uint32_t* parent;       // N or nullptr (world = local)
    const float4* parent_world;   // parent level world, 4 columns per node
    uint32_t num_parents;
    const float4* sphere;         // N
    const uint32_t* geometry;     // N
    const uint32_t* offsets;      // S + 1
    const uint32_t* tile_start;   // per leaf tile: start of the region holding its last drawable
    const uint2* tile_region;     // per leaf tile: regions of its first and last drawable (clamped to S-1)
    uint32_t num_state_sets;
    const uint4* lods;            // G * L
    uint32_t num_geometries;
    uint32_t num_lods;
    uint32_t n;
    float4* world;                // N * 4 (written)
    float4* world_sphere;         // N or nullptr (written)
    uint32_t* cmds;               // N * 5 words
    uint32_t* counts;             // S
    uint32_t* marginal;           // ceil(N/32) or nullptr
    uint32_t* error;              // device-visible error word
    uint32_t off_cap;             // offsets staged in shared memory when S+1 <= off_cap (set by the launcher)
    uint32_t* planes;             // 3 planes of leaf_plane_stride(N) words: visibility, LOD bits 0, 1 (set by the launcher)
    uint32_t* tile_words;         // one word per leaf tile (set by the launcher)
    ShardPlacement shard;         // sharded pass: command placement (dst_base null otherwise)
    ViewConst view;
};

// Sphere-only cull of one view (batched form): inputs are world spheres.
struct ViewJob {
    const float4* world_sphere;
    const uint32_t* geometry;
    const uint32_t* offsets;
    const uint4* lods;
    uint32_t* cmds;
    uint32_t* counts;
    uint32_t* marginal;
    const uint32_t* tile_start;   // the scene's per-tile region starts (tiles of kLeafTile drawables)
    const uint2* tile_region;     // the scene's per-tile first and last regions (tiles of kLeafTile drawables)
    uint32_t n;
    uint32_t num_state_sets;
    uint32_t num_geometries;
    uint32_t num_lods;
    uint32_t first_item;          // first global work item of this view
    uint32_t num_tiles;
    uint32_t pad[4];
    ViewConst view;
};

constexpr int kLeafThreads = 256;
constexpr int kLeafIpt = 8;
constexpr int kLeafTile = kLeafThreads * kLeafIpt;
constexpr int kLeafWarps = kLeafThreads / 32;
// Write kernels: StateSet offsets staged in shared memory up to this many
// entries.  48 registers give 5 CTAs per SM (the plain instance spills 8
// bytes a thread there, the shard instance nothing); the 40 that 6 CTAs
// allow spill 12 and 28 bytes and measured 1% slower on the deep
// hierarchy; 4 CTAs (56 registers, no spills) measured slower on the plain
// pass.
constexpr uint32_t kWriteOffsetCap = 4096;
constexpr int kWriteCtasPerSm = 5;
constexpr int kPropThreads = 256;

// Internal level: world[i] = parent_world[parent[i]] * local[i].
// staged != 0 asserts non-decreasing parents (bulk copy of the parent run).
// With `after_level_kernel` (the launch just before on `stream` is the
// previous level's propagate_kernel) it is launched as that kernel's
// programmatic dependent.
cudaError_t launch_propagate(const float4* parent_world, uint32_t num_parents, const float4* local,
                             const uint32_t* parent, uint32_t n, float4* world, int staged,
                             uint32_t* error, uint64_t spin_limit_ns, cudaStream_t stream,
                             bool after_level_kernel = false);

// The leading internal levels of a deep hierarchy, folded into one launch:
// levels 1..count whose nodes, with level 0's, number at most
// kFoldMaxNodes.  One CTA bulk-copies all their local matrices, parent
// indices and level 0's world matrices into shared memory and propagates
// level after level there, separated by CTA barriers instead of one grid
// dependency per level.  The cap was measured on the deep-hierarchy scene:
// folding its levels of 2, 24 and 216 nodes saves a launch chain, while a
// level of about 2,000 nodes is faster as a grid of its own.
constexpr uint32_t kFoldMaxNodes = 256;
struct FoldLevel {
    const float4* local;
    const uint32_t* parent;
    float4* world;
    uint32_t n;
    uint32_t pad;
};
struct FoldArgs {
    const float4* world0;         // level 0 (world = local)
    uint32_t n0;
    uint32_t count;               // folded levels: 1..count
    FoldLevel lvl[CADR_MAX_LEVELS - 1];
    uint32_t* error;
    uint64_t limit_ns;
};
cudaError_t launch_small_levels(const FoldArgs& a, cudaStream_t stream);

// Leaf level propagation (+ optional world spheres) without culling.
cudaError_t launch_leaf_propagate(const LeafArgs& a, cudaStream_t stream);

// Plain pass over the leaf level: propagate, transform spheres, cull,
// select LOD, compact per StateSet.  Three launches on `stream`; needs
// s.tile_state for ceil(n / kLeafTile) words and s.planes for
// leaf_plane_words(n).  `after_stream`, when not null, is recorded on
// `stream` between the stream kernel and the tile scan.  With
// `after_level_kernel` (the launch just before on `stream` is the last
// level's propagate_kernel) the stream kernel is launched as its
// programmatic dependent.
cudaError_t launch_leaf_cull(const LeafArgs& a, Scratch& s, cudaStream_t stream, cudaEvent_t after_stream,
                             bool after_level_kernel = false);
constexpr uint32_t kLeafCullLaunches = 3;

// The leaf stage in parts, for the sharded pass: the stream kernel and the
// tile scan (launches 1-2); the per-region visible counts from the planes
// and the tile carries (one launch, a.counts); the write kernel (launch 3)
// with the commands placed by a.shard when a.shard.dst_base is set.
cudaError_t launch_leaf_stream_scan(const LeafArgs& a, Scratch& s, cudaStream_t stream, cudaEvent_t after_stream,
                                    bool after_level_kernel);
cudaError_t launch_leaf_region_counts(const LeafArgs& a, Scratch& s, cudaStream_t stream);
cudaError_t launch_leaf_write(const LeafArgs& a, Scratch& s, cudaStream_t stream, bool after_scan);
// Words of one bit-plane: one per 32 drawables, 64 per tile of kLeafTile
// drawables.  Inside a tile, word 8 w + j holds row j of warp w (drawables
// 256 j + 32 w .. + 31 of the tile), so that the 8 words a warp of the
// write kernel reads are 32 contiguous bytes.
__host__ __device__ constexpr uint64_t leaf_plane_stride(uint64_t n) { return ((n + 2047) / 2048) * 64; }
__host__ __device__ constexpr uint64_t leaf_plane_words(uint64_t n) { return 3 * leaf_plane_stride(n); }

// Batched sphere cull over all (view, tile) items, in one of two forms
// (cadr_tuning.form): kBatchedPersistent, one persistent launch of `grid`
// CTAs with a decoupled lookback (scratch: s.ctl and s.tile_state for the
// items); kBatchedThreeLaunch, classify / per-view tile scan / write with
// tiles of kLeafTile drawables and no waits (scratch: s.planes of
// batched_plane_words words).
constexpr uint32_t kBatchedPersistent = 0, kBatchedThreeLaunch = 1;
cudaError_t launch_batched_cull(const ViewJob* d_jobs, uint32_t num_jobs, uint32_t total_items,
                                Scratch& s, uint32_t* error, uint64_t spin_limit_ns, uint32_t fault,
                                const cadr_tuning& tu, uint32_t grid, cudaStream_t stream);
// Drawables per work item of a tuning.
uint32_t batched_tile(const cadr_tuning& tu);
// Plane words a batch of `total_items` items needs (0 for the persistent form).
uint64_t batched_plane_words(const cadr_tuning& tu, uint64_t total_items);

// Tier A.
cudaError_t launch_process_drawables(uint32_t level, const uint64_t* root,
                                     const cadr_drawable_gpu_data* drawables, uint64_t n,
                                     cadr_draw_indirect_cmd* indirect,
                                     cadr_drawable_pointers* pointers, cudaStream_t stream);

}  // namespace cadr
