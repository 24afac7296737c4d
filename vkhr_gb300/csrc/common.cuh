// common.cuh -- shared definitions of the GB300 backend (context, scratch,
// error plumbing, exact FP32 helpers).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>

#include "../../include/vkhr_cuda.h"

// Device status bits (ctx->d_words[WORD_STATUS]).
enum : unsigned {
    VKHR_DEV_STEPS_OVERFLOW = 1u,   // a segment spans >= 2^24 voxels (the reference never terminates)
    VKHR_DEV_LIST_OVERFLOW = 2u,    // fixed-capacity visit list too small
    VKHR_DEV_TIMEOUT = 4u,          // a bounded device wait gave up
    VKHR_DEV_REPLAY_MISMATCH = 8u,  // a brick replay disagreed with its binning (internal error)
    VKHR_DEV_BAD_INDEX = 16u,       // compositing: a fragment's pixel or a PPLL link outside its array
};

// Slots of the small device word array every context owns.
enum {
    WORD_TOTAL_VISITS = 0,      // voxel visits of the current voxelization
    WORD_BIG_LIST = 1,          // brick path: bricks above the shared-memory capacity
    WORD_BIG_QUEUE = 2,         // brick path: next entry of that list
    WORD_STATUS = 3,            // VKHR_DEV_* bits
    WORD_BRICK_CURSOR = 4,      // brick path: allocation cursor of the visit list
    WORD_MAX_BRICK_VISITS = 5,  // brick path: largest brick
    WORD_BHEAVY_COUNT = 6,      // brick path: crowded voxels up to kCrowdWarpMax visits (listed from the front)
    WORD_HKEYS_CURSOR = 7,      // brick path: key scratch cursor (crowded voxels, bricks above kBrickCap)
    WORD_BRICK_QUEUE = 8,       // brick path: next entry of the occupied-brick list
    WORD_BRICK_LIST = 9,        // brick path: occupied bricks resolved in shared memory
    WORD_BHEAVY_BIG = 10,       // brick path: crowded voxels above kCrowdWarpMax visits (listed from the back)
    WORD_DIRECT_OVERFLOW = 11,  // one-walk call: a brick outgrew its fixed slice (the fill pass lays it out)
    WORD_LIGHT_LIST = 12,       // brick path: bricks of up to kLightBrick visits (a warp each)
    WORD_LIGHT_QUEUE = 13,      // brick path: next entry of that list
    WORD_UNCERT_COUNT = 14,     // brick path: uncertified voxels handed to the crowded-warp kernel
    WORD_NORM = 15,             // normalize: min, max (2 slots); words below are cleared per voxelization
    WORD_AABB = 17,             // bounding-box scratch (8 slots)
    WORD_RAY_QUEUE = 25,        // batched raymarch: next tile
    WORD_LAYOUT_CURSOR = 26,    // voxelizer: slice cursor of a learned batch layout
    WORD_COUNT = 27
};

// Visit total of an earlier unbudgeted one-style segment voxelization, by
// the call's size (index count, grid, index mode, tangents requested).
struct vkhr_learned_visits {
    uint64_t items;
    int32_t w, h, d, mode;
    uint64_t visits;           // 0: empty slot
};
constexpr int kLearnedSizes = 16;

struct vkhr_ctx {
    int device;
    int sm_count;
    int l2_bytes;              // L2 cache size
    uint32_t direct_cap;       // voxelizer: per-brick slice capacity of one-walk calls (0: not yet known)
    int walk_ctas[2];          // voxelizer: resident CTAs per SM of the one-walk kernel (one style, batch; 0: no limit)
    int smem_per_sm;           // shared memory per SM and reserved per block (bytes)
    int smem_reserved;
    uint4* d_gather;           // strand reduction: the kept strands' (source, destination, vertices)
    uint32_t* comp;            // compositing: per-pixel counts, slice starts, sort queues, fragment keys
    size_t comp_cap;           // (in 32-bit words)
    size_t d_gather_cap;
    void* slots;               // voxelizer: the fixed per-brick slices of one-walk calls
    size_t slots_cap;          // (in 8-byte units)
    uint2* layout;             // voxelizer: learned {first slot, capacity} per brick of a batch's one walk
    size_t layout_cap;         // (in bricks)
    uint64_t layout_shape;     // the batch shape it was learned for (0: none)
    uint32_t layout_bricks;    // bricks of that batch
    uint64_t layout_slots;     // slots its slices span
    // grow-only scratch (capacities in elements)
    uint32_t* brick_runs;      // voxelizer: visits and visit-list cursor per brick (2 x bricks)
    uint32_t* brick_visits;
    uint32_t* brick_cursor;
    size_t brick_cap;
    uint2* items;              // voxelizer: visit entries (key, local voxel), grouped by brick
    size_t items_cap;
    uint32_t* brick_list;      // voxelizer: occupied bricks of the shared-memory path
    size_t brick_list_cap;
    float4* pair_tan;          // voxelizer: per index pair, the tangent of its first vertex
    size_t pair_tan_cap;
    uint32_t* hkeys;           // voxelizer: key scratch (crowded voxels, bricks above the shared-memory cap)
    size_t hkeys_cap;
    uint4* hdesc;              // voxelizer: crowded, then uncertified voxels (voxel, key offset, count, job)
    size_t hdesc_cap;
    void* d_jobs;              // voxelizer: device job table of the current batch
    size_t jobs_cap;           // in bytes
    void* h_jobs;              // pinned staging of the job table
    cudaEvent_t jobs_ev;       // recorded after the staging was copied out
    uint64_t visit_budget;     // segment mode: fixed visit capacity (0 = size from the counted total)
    vkhr_learned_visits learned[kLearnedSizes]; // segment mode without a budget: earlier calls' visits
    int learned_next;          // slot the next new size replaces
    int live_graphs;           // frame graphs holding pointers into this context's scratch
    void* d_rjobs;             // raymarch: device job table of the current batch
    size_t rjobs_cap;          // in bytes
    void* h_rjobs;             // pinned staging of the raymarch job table
    cudaEvent_t rjobs_ev;      // recorded after the staging was copied out
    int ray_variant[3][2];     // raymarch packet variant per (density format, tangent format)
    float* g_acc;              // adjoint: per-pixel gradient of the accumulated density
    size_t g_acc_cap;
    uint32_t* occ;             // raymarch brick-occupancy bitmap
    size_t occ_cap;            // in 32-bit words
    cudaArray_t tex_array;     // raymarch, texture-unit variant: the density copied into a 3D array
    cudaTextureObject_t tex_obj; // (LINEAR filter, border 0) and its texture object
    int tex_res[3], tex_fmt;   // the array's extent and density format
    cudaArray_t gat_array;     // raymarch, gather variant: the density's slices tiled into a 2D array
    cudaTextureObject_t gat_obj; // (POINT filter, element type, border 0) and its texture object
    cudaSurfaceObject_t gat_surf; // its surface, when the array could be made writable (else 0: staged copies)
    int gat_res[3], gat_fmt, gat_shift; // the grid it holds, its density format, log2 tiles per row
    void* gat_stage;           // linear staging of the tiled slices
    size_t gat_stage_cap;      // in bytes
    unsigned long long* d_words;
    unsigned long long* h_words; // pinned mirror
    cudaEvent_t ev;
    // side stream for kernels that overlap the main chain (fork/join by events,
    // so a captured call captures both streams)
    cudaStream_t side;
    cudaEvent_t fork_ev, join_ev;
    unsigned long long launches; // kernels this context has launched
    // kernel tracer (vkhr_set_profiling): an event pair around every launch
    int profiling;
    int prof_n;
    cudaEvent_t* prof_ev;        // 2 * kProfileMax events
    const char** prof_name;      // kProfileMax kernel names
    char last_error[512];
};

constexpr int kProfileMax = 4096;
constexpr size_t kJobTableBytes = 64 * 1024;  // pinned staging of a voxelizer batch's job table
constexpr size_t kRayTableBytes = 256 * 1024; // pinned staging of a raymarch batch's job table

void vkhr_prof_begin(vkhr_ctx* ctx, const char* name, cudaStream_t st);
void vkhr_prof_end(vkhr_ctx* ctx, cudaStream_t st);

// Launch bookkeeping: every kernel launch of the library goes through this.
#define VKHR_LAUNCH(ctx, kernel, grid, block, smem, stream, ...)                                  \
    do {                                                                                           \
        if ((ctx)->profiling) vkhr_prof_begin((ctx), #kernel, (stream));                           \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                                \
        if ((ctx)->profiling) vkhr_prof_end((ctx), (stream));                                      \
        ++(ctx)->launches;                                                                         \
    } while (0)

#define VKHR_CUDA_TRY(ctx, call)                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return vkhr_fail_cuda((ctx), e_, #call, __FILE__, __LINE__);       \
    } while (0)

vkhr_status vkhr_fail(vkhr_ctx* ctx, vkhr_status s, const char* msg);
// The side stream waits for the work queued so far on st / st waits for the
// work queued so far on the side stream.
vkhr_status vkhr_fork_side(vkhr_ctx* ctx, cudaStream_t st);
vkhr_status vkhr_join_side(vkhr_ctx* ctx, cudaStream_t st);
vkhr_status vkhr_fail_cuda(vkhr_ctx* ctx, cudaError_t e, const char* what, const char* file, int line);

// Grow-only device buffer; contents are not preserved on growth.  While a
// frame graph of the context exists, a buffer that would have to grow is
// refused (VKHR_ERR_CAPACITY): the graph holds its address.
vkhr_status vkhr_reserve(vkhr_ctx* ctx, void** ptr, size_t* cap_elems, size_t need_elems, size_t elem_bytes);

// One-style segment voxelization that reads its visit total back (into
// *visits) whatever the context has learned; the context's budget is kept.
vkhr_status vkhr_voxelize_counted(vkhr_ctx* ctx, const vkhr_voxel_job* job, void* stream, uint64_t* visits);

static inline unsigned vkhr_blocks(size_t n, unsigned threads)
{
    size_t b = (n + threads - 1) / threads;
    return (unsigned)(b == 0 ? 1 : b);
}

// ---- exact FP32 helpers (no contraction, round-to-nearest) ---------------------
// glm::min(x, y) = y < x ? y : x and glm::max(x, y) = x < y ? y : x.
__device__ __forceinline__ float glm_min(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float glm_max(float x, float y) { return (x < y) ? y : x; }
