/*
 * vkhr_cuda.h -- C ABI of the GB300 (sm_103a) backend for vkhr's volumetric
 * level-of-detail path: the strand-density voxelizer and the volume raymarcher.
 *
 * Every entry point takes plain device pointers and sizes and returns a
 * vkhr_status; nothing throws across this boundary.  All work is ordered on
 * the caller's CUDA stream (passed as `void*`, i.e. a cudaStream_t; NULL is
 * the legacy default stream).  The library owns only its scratch memory
 * (held by the context); inputs and outputs are always caller-owned.
 *
 * Reference interfaces replaced (paths inside the vkhr project):
 *   vkhr::HairStyle::generate_bounding_box / get_bounding_box
 *                                        src/vkhr/scene_graph/hair_style.cc:215-255
 *   vkhr::HairStyle::generate_tangents   src/vkhr/scene_graph/hair_style.cc:171-194
 *   vkhr::HairStyle::generate_indices    src/vkhr/scene_graph/hair_style.cc:196-213
 *   vkhr::HairStyle::voxelize_vertices   src/vkhr/scene_graph/hair_style.cc:257-294
 *   vkhr::HairStyle::voxelize_segments   src/vkhr/scene_graph/hair_style.cc:296-342
 *   vkhr::HairStyle::Volume::normalize   src/vkhr/scene_graph/hair_style.cc:344-357
 *   vulkan::Volume::draw + volume.frag   src/vkhr/rasterizer/volume.cc:104-112,
 *                                        share/shaders/volumes/volume.frag:31-103
 *   vulkan::LinkedList::resolve          src/vkhr/rasterizer/linked_list.cc:21-41,
 *     + resolve.comp                     share/shaders/transparency/resolve.comp:15-101
 */
#ifndef VKHR_CUDA_H
#define VKHR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VKHR_CUDA_ABI_VERSION 2

typedef enum vkhr_status {
    VKHR_OK = 0,
    VKHR_ERR_INVALID_ARG = 1,      /* null pointer, bad size, bad enum value      */
    VKHR_ERR_DEGENERATE_AABB = 2,  /* a zero (or NaN) extent: voxel size would be 0 */
    VKHR_ERR_OOM = 3,              /* scratch allocation failed                   */
    VKHR_ERR_CUDA = 4,             /* a CUDA runtime call failed (see last error) */
    VKHR_ERR_TIMEOUT = 5,          /* a bounded device wait ran out               */
    VKHR_ERR_NAN_INPUT = 6,        /* non-finite vertex coordinates               */
    VKHR_ERR_CAPACITY = 7,         /* fixed-capacity scratch was too small        */
    VKHR_ERR_NOT_SUPPORTED = 8     /* valid request this build does not implement */
} vkhr_status;

/* vkhr::AABB (include/vkhr/scene_graph/hair_style.hh:16-21), same layout:
 * origin = min corner, size = max - min, radius = |size|, volume = x*y*z.   */
typedef struct vkhr_aabb {
    float origin[3];
    float radius;
    float size[3];
    float volume;
} vkhr_aabb;

/* How the linear voxel index is formed.  The reference evaluates
 * `voxel.x + voxel.y*width + voxel.z*width*height` in FP32
 * (hair_style.cc:276, :321), which is exact only below 2^24 voxels.
 *  REF_FP32 reproduces that expression bit for bit (identical to EXACT at
 *           <= 2^24 voxels, i.e. up to 256^3); visits whose FP32 index falls
 *           outside [0, w*h*d) are dropped (the reference writes out of bounds).
 *  EXACT    integer indexing; visits with a negative coordinate are dropped. */
typedef enum vkhr_index_mode {
    VKHR_INDEX_REF_FP32 = 0,
    VKHR_INDEX_EXACT = 1
} vkhr_index_mode;

/* Density texel formats the raymarcher samples. */
typedef enum vkhr_density_format {
    VKHR_DENSITY_U8_UNORM = 0,  /* reference: R8_UNORM of normalize()d densities */
    VKHR_DENSITY_U32_COUNT = 1, /* raw uint32 strand counts, sampled as floats   */
    VKHR_DENSITY_F32 = 2        /* FP32 density                                  */
} vkhr_density_format;

/* Tangent texel formats. */
typedef enum vkhr_tangent_format {
    VKHR_TANGENT_I8_SNORM = 0,  /* reference: R8G8B8A8_SNORM, 4 bytes per voxel */
    VKHR_TANGENT_F32X4 = 1      /* FP32 x4, 16 bytes per voxel                   */
} vkhr_tangent_format;

/* Shading models of the Params UBO (kajiya-kay.glsl:4, approximate_deep_shadows.glsl:4,
 * local_ambient_occlusion.glsl:4). */
enum {
    VKHR_SHADING_KAJIYA_KAY = 0,
    VKHR_SHADING_ADSM = 2,
    VKHR_SHADING_LAO = 3
};

/* Renderer::Type (include/vkhr/renderer.hh:13-17).  lod() of scheme.glsl:7-11
 * is 0 for the rasterizer, 1 for the raymarcher and the smoothstep blend for
 * every other value (the ray tracer's and the hybrid's). */
enum {
    VKHR_RENDERER_RASTERIZER = 0,
    VKHR_RENDERER_RAY_TRACER = 1,
    VKHR_RENDERER_RAYMARCHER = 2,
    VKHR_RENDERER_HYBRID_LOD = 3
};

/* Every scalar the raymarch reads.  Field groups mirror the reference UBOs:
 *   camera  -- Camera UBO (share/shaders/scene_graph/camera.glsl:4-11),
 *              matrices column-major exactly as glm::mat4 stores them;
 *   light   -- Lights UBO entry 0 (share/shaders/scene_graph/lights.glsl:4-13);
 *   strand  -- Strand UBO (share/shaders/strands/strand.glsl:8-16);
 *   params  -- Params UBO (share/shaders/scene_graph/params.glsl:7-33);
 *   fixed   -- literals of volume.frag (:78 thickness 11.0, :86 AO kernel 2);
 *   ext     -- knobs beyond the reference; their defaults reduce to it. */
typedef struct vkhr_raymarch_params {
    int32_t width, height;              /* framebuffer size in pixels                */

    float view[16];                     /* camera.view                               */
    float projection[16];               /* camera.projection (Vulkan y-flip applied) */
    float camera_position[3];           /* camera.position                           */
    float look_at_distance;             /* camera.look_at_distance                   */

    float light_origin[3];              /* lights[0].origin                          */
    float light_intensity[3];           /* lights[0].intensity                       */

    vkhr_aabb volume_bounds;            /* volume_bounds                             */
    int32_t volume_resolution[3];       /* volume_resolution                         */
    float hair_color[3];                /* hair_color                                */
    float hair_alpha;                   /* hair_alpha                                */
    float hair_exponent;                /* hair_exponent                             */

    int32_t shading_model;              /* shading_model                             */
    int32_t deep_shadows_on;            /* deep_shadows_on (YES = 1)                 */
    float isosurface;                   /* isosurface                                */
    float raycast_steps;                /* raycast_steps                             */
    float occlusion_radius;             /* occlusion_radius                          */
    float ao_exponent;                  /* ao_exponent                               */
    float ao_max;                       /* ao_max                                    */
    float magnified_distance;           /* magnified_distance                        */
    int32_t renderer;                   /* renderer                                  */
    float minified_distance;            /* minified_distance                         */

    float shadow_thickness;             /* 11.0 in volume.frag:78                    */
    float ao_kernel_size;               /* 2 in volume.frag:86                       */

    float shadow_steps;                 /* ext: <= 0 means raycast_steps (reference) */
    float kd;                           /* ext: diffuse scale, 1 = reference         */
    int32_t density_format;             /* vkhr_density_format                       */
    int32_t tangent_format;             /* vkhr_tangent_format                       */

    float spec_exponent2;               /* ext: second lobe's exponent; <= 0 = none  */
    float spec_shift[2];                /* ext: tangent shift of lobe 1 / lobe 2     */
    int32_t ao_directions;              /* ext: 0 = the ao_kernel_size^3 cube, else
                                           that many directions (1..32)             */
} vkhr_raymarch_params;

/* The extension knobs, exactly (all zero: the reference's shading):
 *
 * Dual-lobe Kajiya-Kay.  With T the normalised surface tangent, L and E as in
 * kajiya-kay.glsl:7-24 (E points from the camera to the surface), V = -E and
 * N = normalize(V - (T.V) T) (the unit direction towards the camera
 * perpendicular to the strand; N = 0 when T is parallel to E), lobe j uses
 * the shifted tangent T_j = normalize(T + spec_shift[j] * N):
 *   spec_j  = max(cos(T_j,L) cos(T_j,E) + sin(T_j,L) sin(T_j,E), 0)^p_j,
 *   shading = kd * sin(T,L) * hair_color + spec_1 * light_intensity
 *             + spec_2 * light_intensity * hair_color        (second lobe),
 * p_1 = hair_exponent, p_2 = spec_exponent2; the second lobe exists when
 * spec_exponent2 > 0.  A positive shift turns the strand towards the viewer
 * by atan(shift).
 *
 * Directional ambient occlusion.  ao_directions = n > 0 replaces the
 * ao_kernel_size^3 cube of local_ambient_occlusion.glsl:9-30 by n taps at
 *   s + d_i * (occlusion_radius * sqrt(3)) * voxel_size   (per axis),
 * d_i the Fibonacci-sphere directions (y the polar axis):
 *   y_i = 1 - (2i + 1) / n,  r_i = sqrt(1 - y_i^2),  phi_i = i * pi * (3 - sqrt(5)),
 *   d_i = (r_i cos phi_i, y_i, r_i sin phi_i),
 * and occlusion = (1 - sum_i min(density_i, ao_max) / n)^ao_exponent.  The
 * radius factor sqrt(3) puts the taps at the distance of the reference's
 * 8-tap cube (kernel 2), whose taps are the 8 directions (+-1, +-1, +-1)/sqrt(3). */

/* Opaque library context: one per host thread (or externally synchronised).
 * It pins a device and owns grow-only scratch buffers. */
typedef struct vkhr_ctx vkhr_ctx;

/* ---- context ------------------------------------------------------------- */
vkhr_status vkhr_create(int device, vkhr_ctx** out_ctx);
vkhr_status vkhr_destroy(vkhr_ctx* ctx);
const char* vkhr_status_string(vkhr_status status);
/* Text of the last failure seen by this context (never NULL). */
const char* vkhr_last_error(const vkhr_ctx* ctx);
int vkhr_abi_version(void);
/* Kernel tracer: with profiling on, every kernel launch is bracketed by a
 * CUDA event pair on its own stream (the reference brackets each pass with
 * Vulkan timestamp queries, src/vkpp/query.cc:124-137).  Enabling clears the
 * record; vkhr_profile_read waits for record `index` and returns its kernel
 * name and duration in milliseconds.  At most 4096 launches are recorded. */
vkhr_status vkhr_set_profiling(vkhr_ctx* ctx, int enable);
int vkhr_profile_count(const vkhr_ctx* ctx);
vkhr_status vkhr_profile_read(vkhr_ctx* ctx, int index, const char** name, float* ms);
/* Number of kernels this context has launched so far (instrumentation). */
uint64_t vkhr_launch_count(const vkhr_ctx* ctx);
/* sizeof of the ABI structures as this library was compiled (layout checks). */
size_t vkhr_sizeof_aabb(void);
size_t vkhr_sizeof_raymarch_params(void);
size_t vkhr_sizeof_voxel_job(void);
size_t vkhr_sizeof_raymarch_job(void);

/* ---- device memory helpers ---------------------------------------------------
 * So that a host without the CUDA toolkit (the reference's C++17 code) can
 * stage its std::vector data: plain cudaMalloc / cudaFree / cudaMemcpyAsync
 * on the context's device.  Copies are stream-ordered; vkhr_sync waits. */
vkhr_status vkhr_malloc(vkhr_ctx* ctx, size_t bytes, void** d_out);
vkhr_status vkhr_free(vkhr_ctx* ctx, void* d_ptr);
vkhr_status vkhr_upload(vkhr_ctx* ctx, void* d_dst, const void* h_src, size_t bytes, void* stream);
vkhr_status vkhr_download(vkhr_ctx* ctx, void* h_dst, const void* d_src, size_t bytes, void* stream);
vkhr_status vkhr_sync(vkhr_ctx* ctx, void* stream);

/* ---- strand data preparation ----------------------------------------------
 * Replaces HairStyle::generate_bounding_box + get_bounding_box
 * (hair_style.cc:215-255): min/max start at (0,0,0), so the box always holds
 * the world origin.  Writes the AABB to *out_bounds (host memory) and
 * synchronises the stream.  NaN/Inf vertices give VKHR_ERR_NAN_INPUT. */
vkhr_status vkhr_bounding_box(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count,
                              vkhr_aabb* out_bounds, void* stream);

/* Replaces HairStyle::generate_tangents (hair_style.cc:171-194).  Strand s has
 * h_segments[s] segments (the HAIR `segments` array; strand_count entries,
 * host memory) and segments+1 vertices; the last vertex repeats the previous
 * tangent.  d_tangents receives vertex_count float3 (12 bytes each). */
vkhr_status vkhr_generate_tangents(vkhr_ctx* ctx, const float* d_vertices, const uint16_t* h_segments,
                                   uint32_t strand_count, float* d_tangents, void* stream);

/* Replaces HairStyle::generate_indices (hair_style.cc:196-213): two uint32 per
 * segment, skipping the last vertex of every strand.  d_indices receives
 * 2 * sum(segments) entries. */
vkhr_status vkhr_generate_indices(vkhr_ctx* ctx, const uint16_t* h_segments, uint32_t strand_count,
                                  uint32_t* d_indices, void* stream);

/* ---- voxelization ----------------------------------------------------------
 * Outputs (all device memory, x fastest, then y, then z):
 *   d_counts     uint32 per voxel: the exact number of visits (never saturates);
 *   d_densities  uint8 per voxel: HairStyle::Volume::densities, i.e.
 *                min(count, 255) (optional, may be NULL);
 *   d_tangents   int8 x4 per voxel: HairStyle::Volume::tangents, bit-exact
 *                including the reference's serial summation order and its
 *                stop-at-255 rule (optional, may be NULL; needs d_tangent_in).
 * d_vertices / d_tangent_in are float3 arrays (12-byte stride, glm::vec3).
 * bounds is host memory.  Scratch comes from the context and grows on
 * demand (a growth allocates, which synchronises the device).
 *
 * Host waits.  Vertex mode never waits on the host.  Segment mode sizes its
 * visit list from the number of voxel visits:
 *   - with a visit budget (vkhr_set_visit_budget) from the budget: no wait;
 *   - without one, a one-style call at a size (index count, grid, index mode,
 *     tangents or not) that this context has voxelized before sizes it from
 *     twice that earlier call's visits: no wait.  A call whose visits exceed
 *     that records VKHR_ERR_CAPACITY, which vkhr_check_status reports (its
 *     outputs are then incomplete); the context then forgets the sizes it
 *     learned, and the next call at each size counts again;
 *   - otherwise (the first call at a size, and every batch of two or more
 *     styles) the call reads its visit total back: one 8-byte copy and a
 *     wait for `stream`.
 * A call under stream capture must not need the read-back. */

/* Replaces HairStyle::voxelize_vertices (hair_style.cc:257-294). */
vkhr_status vkhr_voxelize_vertices(vkhr_ctx* ctx, const float* d_vertices, const float* d_tangent_in,
                                   uint32_t vertex_count, const vkhr_aabb* bounds,
                                   int32_t width, int32_t height, int32_t depth, int32_t index_mode,
                                   uint32_t* d_counts, uint8_t* d_densities, int8_t* d_tangents,
                                   void* stream);

/* Replaces HairStyle::voxelize_segments (hair_style.cc:296-342).  d_indices
 * holds index_count uint32 (pairs; an odd trailing index is ignored, as the
 * reference's `i < indices.size() - 1` loop does). */
vkhr_status vkhr_voxelize_segments(vkhr_ctx* ctx, const float* d_vertices, const float* d_tangent_in,
                                   const uint32_t* d_indices, uint64_t index_count, const vkhr_aabb* bounds,
                                   int32_t width, int32_t height, int32_t depth, int32_t index_mode,
                                   uint32_t* d_counts, uint8_t* d_densities, int8_t* d_tangents,
                                   void* stream);

/* One style of a batched voxelization: the arguments of vkhr_voxelize_vertices
 * (item_count = vertex_count, d_indices unused) or vkhr_voxelize_segments
 * (item_count = index_count). */
typedef struct vkhr_voxel_job {
    const float* d_vertices;
    const float* d_tangent_in;
    const uint32_t* d_indices;
    uint64_t item_count;
    vkhr_aabb bounds;
    int32_t width, height, depth;
    int32_t index_mode;
    uint32_t* d_counts;
    uint8_t* d_densities;
    int8_t* d_tangents;
} vkhr_voxel_job;

/* Voxelizes job_count (1..256) styles with one launch per phase: the
 * per-style loop of the reference's loader (hair_style.cc:75, once per
 * HairStyle) fused into one call.  Results per job are those of the
 * single-style entry point; either every job requests d_tangents or none.
 * No reference counterpart as a single call. */
vkhr_status vkhr_voxelize_batched(vkhr_ctx* ctx, int32_t segments, const vkhr_voxel_job* jobs, int32_t job_count,
                                  void* stream);

/* Segment voxelization normally reads its visit total back to size the visit
 * list.  A nonzero budget fixes that capacity instead (max_visits < 2^32), so
 * the call never waits on the host and can be captured into a CUDA graph
 * after one uncaptured call at the same sizes; a batch that needs more visits
 * reports VKHR_ERR_CAPACITY from vkhr_check_status.  0 restores the default.
 * No reference counterpart. */
vkhr_status vkhr_set_visit_budget(vkhr_ctx* ctx, uint64_t max_visits);

/* Resident CTAs per SM of the one-walk segment kernel (the counting walk that
 * also writes each visit into its brick's slice), no reference counterpart:
 * 0 = as many as registers allow (8), else 1..8.  Fewer resident walks
 * queue less on the per-brick counters whose returning atomics reserve the
 * slices.  which: 0 = one-style calls, 1 = batches.  Default: 0 for both.
 * The results do not depend on it. */
vkhr_status vkhr_set_voxelize_walk(vkhr_ctx* ctx, int32_t which, int32_t ctas_per_sm);

/* Autotuner for the above (no reference counterpart): voxelizes the segment
 * jobs (one-style calls for job_count == 1, else a batch) once without a
 * budget (counting its visits, learning the one-walk slices), then times
 * each residency of {0, 2, 3, 4, 5, 6} (one warm-up and three timed runs
 * each) under the context's visit budget, or the counted visits + 25% +
 * 4096 when it has none (restored afterwards); keeps the fastest for that
 * kind of call and writes it to *chosen and, when ms is not NULL, each
 * choice's median time (VKHR_WALK_CHOICES floats, in that order).  The jobs'
 * outputs receive the voxelization.  Synchronises the stream. */
#define VKHR_WALK_CHOICES 6
vkhr_status vkhr_autotune_voxelize(vkhr_ctx* ctx, const vkhr_voxel_job* jobs, int32_t job_count, int32_t* chosen,
                                   float* ms, void* stream);

/* Waits for the stream and reports errors that kernels recorded on the device
 * since the last report (e.g. a capacity overflow, a fragment outside the
 * image); reporting clears them.  A segment voxelization that reads its
 * visit total back reports them the same way. */
vkhr_status vkhr_check_status(vkhr_ctx* ctx, void* stream);

/* Replaces HairStyle::Volume::normalize (hair_style.cc:344-357): u8 min-max
 * rescale in place.  A constant volume (max == min) maps to 0, where the
 * reference divides by zero. */
vkhr_status vkhr_normalize_densities(vkhr_ctx* ctx, uint8_t* d_densities, uint64_t voxel_count, void* stream);
/* (d_densities must be 16-byte aligned, as cudaMalloc returns.) */

/* Filters of Volume::downsample (hair_style.hh:228-257), which takes any
 * functor of the 2x2x2 neighbourhood; the ABI offers these. */
typedef enum vkhr_downsample_filter {
    VKHR_FILTER_MAX = 0,      /* max of the 8 densities              */
    VKHR_FILTER_MIN = 1,      /* min of the 8 densities              */
    VKHR_FILTER_MEAN = 2,     /* floor(sum / 8)                      */
    VKHR_FILTER_SUM = 3       /* min(sum, 255)                       */
} vkhr_downsample_filter;

/* Replaces HairStyle::Volume::downsample (hair_style.hh:228-257): u8
 * densities of a width x height x depth grid reduced 2x2x2 into a
 * (width/2) x (height/2) x (depth/2) grid.  The dimensions must be even (for
 * odd ones the reference reads past rows and past the end of the grid). */
vkhr_status vkhr_downsample_densities(vkhr_ctx* ctx, const uint8_t* d_in, int32_t width, int32_t height,
                                      int32_t depth, int32_t filter, uint8_t* d_out, void* stream);

/* ---- raymarch ---------------------------------------------------------------
 * Replaces the Vulkan draw of the volume proxy cube (volume.cc:104-112) and
 * the fragment shader volume.frag:31-103 with its includes.  One ray per
 * pixel centre whose ray enters the AABB from outside (the front faces the
 * reference rasterizes with back-face culling); a camera inside the box
 * covers no pixel, as in the reference.
 *   d_density   density texels in params->density_format;
 *   d_tangent   tangent texels in params->tangent_format;
 *   d_depth_in  optional depth buffer (width*height floats, NULL = cleared 1.0);
 *   d_rgba      width*height float4: (shading*occlusion, coverage) clamped
 *               to [0,1] as packUnorm4x8 does (ppll.glsl:32); 0 where no
 *               fragment survives (discarded or not covered);
 *   d_depth_out optional width*height floats: fragment depth, 1.0 elsewhere. */
vkhr_status vkhr_raymarch(vkhr_ctx* ctx, const vkhr_raymarch_params* params,
                          const void* d_density, const void* d_tangent, const float* d_depth_in,
                          float* d_rgba, float* d_depth_out, void* stream);

/* Ray-packet variants of vkhr_raymarch: 0 = 8x4-pixel warp tiles (default),
 * 1 = 16x2, 2 = 4x8, 3 = 8x4 with 8 resident CTAs per SM (fewer registers),
 * 4 = 8x4 tiles whose primary march reads density texels from shared memory,
 * each occupied 8^3 brick a warp's rays need staged by one TMA tensor copy
 * (used where TMA can address the grid: a 16-byte aligned base and a row
 * pitch of whole 16 bytes; variant 0 elsewhere).  Variants 0-4 compute the
 * same pixels, bit for bit.  5 = 8x4 tiles sampling the density through the
 * texture unit: the call copies it into a 3D array of the context (LINEAR
 * filtering, border 0) and the hardware filters it with 8-bit weights, so its
 * pixels differ from the others by that filter's precision; u8 and FP32
 * densities only (variant 0 for counts).  6 = variant 5's texture for the
 * shading's samples only (deep-shadow march and ambient-occlusion taps),
 * while the isosurface search reads the texels in memory as variant 0 does.
 * The autotuner tries neither 5 nor 6.  7 = 8x4 tiles reading the texels
 * through the texture unit's 2x2 gathers (exact values, no filtering) from a
 * 2D array of the grid's z slices, tiled and framed by zeros, that the call
 * copies the density into; the software trilinear filters them, so its
 * pixels are variant 0's, bit for bit (variant 0 where the tiled slices
 * exceed the gather limits).  8 / 9 / 10 = ray groups, the steps-per-thread
 * knob: 4 / 2 / 8 lanes march each pixel's ray, taking as many consecutive
 * samples of its primary march, its shadow march and its occlusion taps at
 * once and replaying them in order (4x2 / 4x4 / 2x2 pixels per warp);
 * variant 0's pixels, bit for bit.  They pay where few rays march far (a
 * distant volume's small footprint) and lose where many rays fill the GPU. */
#define VKHR_RAYMARCH_VARIANTS 11

/* Autotuner (no reference counterpart): times each variant of vkhr_raymarch
 * that computes the reference's pixels (0-4 and 7-10) on these inputs (one warm-up
 * and three timed runs each, d_rgba receiving the image) and keeps the
 * fastest in the context for params' texel formats; later vkhr_raymarch
 * calls with those formats use it.  Writes the choice to *chosen and, when
 * variant_ms is not NULL, the median time of each variant
 * (VKHR_RAYMARCH_VARIANTS floats; 0 for variants 5 and 6, not timed).  Synchronises
 * the stream. */
vkhr_status vkhr_autotune_raymarch(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const void* d_density,
                                   const void* d_tangent, float* d_rgba, int32_t* chosen, float* variant_ms,
                                   void* stream);

/* Selects a variant for a pair of texel formats without timing. */
vkhr_status vkhr_set_raymarch_variant(vkhr_ctx* ctx, int32_t density_format, int32_t tangent_format, int32_t variant);

/* One view of a batched raymarch: its parameters (width x height is the whole
 * view the camera projects to), its volume, and the region [x0, x0 + w) x
 * [y0, y0 + h) of the view to render.  Outputs use the region's layout: pixel
 * (x0 + i, y0 + j) of the view lands at d_rgba[j * pitch + i] (float4) and
 * d_depth_out[j * pitch + i]; d_depth_in (optional) is read the same way, so
 * regions of several views can be packed into one atlas. */
typedef struct vkhr_raymarch_job {
    vkhr_raymarch_params params;
    const void* d_density;
    const void* d_tangent;
    const float* d_depth_in;
    float* d_rgba;
    float* d_depth_out;
    int32_t x0, y0, w, h;
    int32_t pitch;
    int32_t reserved;
} vkhr_raymarch_job;

/* Raymarches job_count (1..256) views in one persistent launch fed by a
 * device tile queue (the per-style Volume::draw calls of
 * Rasterizer::strand_dvr, rasterizer.cc, as one call).  Each pixel equals the
 * one vkhr_raymarch computes for the same view.  All jobs share one density
 * and one tangent format.  After one uncaptured call at the same sizes the
 * call can be captured into a CUDA graph; the graph then re-reads the job
 * table staged in the context, so the context makes no other batched
 * raymarch while that graph is in use.  No reference counterpart as a single
 * call. */
vkhr_status vkhr_raymarch_batched(vkhr_ctx* ctx, const vkhr_raymarch_job* jobs, int32_t job_count, void* stream);

/* Screen footprint of params' volume: the smallest pixel rectangle (x0, y0,
 * w, h) outside which vkhr_raymarch writes only background (rgba 0, depth
 * 1.0), with 2 pixels of margin; the whole view when a box corner is behind
 * the camera; w = h = 0 when the box is off screen.  Host-only. */
vkhr_status vkhr_raymarch_footprint(const vkhr_raymarch_params* params, int32_t rect[4]);

/* ---- differentiable path ----------------------------------------------------
 * No reference counterpart: gradients of an image loss with respect to an FP32
 * density volume (VKHR_DENSITY_F32), an FP32 tangent field (VKHR_TANGENT_F32X4,
 * w ignored), kd and the specular exponents, and -- through the trilinear splat below --
 * the strand vertex positions.  The forward is the raymarch of vkhr_raymarch
 * (same results, bit for bit); the isosurface point, the early exit and the
 * zero tests are constants of the derivative, the clamps of the output pass
 * gradient only strictly inside (0, 1).  No depth buffer. */

/* Bytes of the per-ray tape of vkhr_raymarch_train: 32 bytes of state per
 * pixel plus the march's t every checkpoint_interval iterations (0 for
 * invalid parameters). */
size_t vkhr_raymarch_tape_bytes(const vkhr_raymarch_params* params, int32_t checkpoint_interval);

/* vkhr_raymarch that also records the tape (16-byte aligned, caller-owned)
 * vkhr_raymarch_adjoint replays. */
vkhr_status vkhr_raymarch_train(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const float* d_density,
                                const float* d_tangent, float* d_rgba, float* d_depth_out, void* d_tape,
                                size_t tape_bytes, int32_t checkpoint_interval, void* stream);

/* Adds dL/d(density), dL/d(tangent) (float4 per voxel, w left alone) and
 * [dL/d kd, dL/d hair_exponent, dL/d spec_exponent2] (three doubles; the last
 * stays 0 without a second lobe) to the caller's buffers, given
 * dL/d(rgba) (float4 per pixel) and the tape of the training forward on the
 * same inputs.  The primary march is replayed from the tape's checkpoints,
 * one thread per ray segment of checkpoint_interval iterations. */
vkhr_status vkhr_raymarch_adjoint(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const float* d_density,
                                  const float* d_tangent, const void* d_tape, int32_t checkpoint_interval,
                                  const float* d_grad_rgba, float* d_grad_density, float* d_grad_tangent,
                                  double* d_grad_params, void* stream);

/* Continuous trilinear-splat voxelization: every vertex adds its trilinear
 * weights (in the raymarch's texel convention: texel centres at
 * origin + (i + 0.5) * size / N) to the FP32 density (accumulated into). */
vkhr_status vkhr_splat_vertices(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count, const vkhr_aabb* bounds,
                                int32_t width, int32_t height, int32_t depth, float* d_density, void* stream);

/* dL/d(vertex) (float3 per vertex, written) of the splat, given dL/d(density). */
vkhr_status vkhr_splat_vertices_adjoint(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count,
                                        const vkhr_aabb* bounds, int32_t width, int32_t height, int32_t depth,
                                        const float* d_grad_density, float* d_grad_vertices, void* stream);

/* Allocation-free raymarch.  No counterpart in the reference: it exists for
 * callers that may not allocate device memory at all -- a real-time frame
 * loop that forbids cudaMalloc (which synchronises the device and takes an
 * unbounded time), or a host engine that owns the whole GPU memory budget and
 * does not let plugins allocate.  Same inputs, outputs and results as
 * vkhr_raymarch, but no context: the raymarch's only scratch (its brick
 * occupancy bitmap) lives in a fixed 128 KiB array inside the library that
 * every device loading the library holds until the process exits.
 *   - Limit: ((w+8)/8) * ((h+8)/8) * ((d+8)/8) <= 1,048,576 occupancy bricks
 *     (volumes up to about 800^3); larger grids return VKHR_ERR_CAPACITY.
 *   - It runs on the current device (cudaSetDevice): the pointers and the
 *     stream must belong to that device.
 *   - The first call on a device looks up the array's device address (and
 *     the SM count).  A lookup that fails returns VKHR_ERR_CUDA and is tried
 *     again by the next call.
 *   - All calls share the one array and it keeps the previous call's bits
 *     (each call clears the part it uses): calls that can overlap on the GPU
 *     (different streams, or different host threads) race; order them.
 *   - Allocates nothing: no cudaMalloc/cudaFree, no allocating library call.
 *   - Status only (no context, so no vkhr_last_error text). */
vkhr_status vkhr_raymarch_static(const vkhr_raymarch_params* params, const void* d_density, const void* d_tangent,
                                 const float* d_depth_in, float* d_rgba, float* d_depth_out, void* stream);

/* Per-frame voxelization feeding the raymarcher without a host round trip:
 * one CUDA graph of a style's voxelization (rasterizer.cc:216-230, the
 * per-frame voxelize pass of the paper), optionally Volume::normalize, the
 * brick-occupancy pass and the raymarch of one view (volume.cc:104-112).
 * Create captures the three calls once; launch replays them on a stream.
 * Between launches the caller rewrites the job's input buffers in place (a
 * hair simulation moving the vertices and tangents); every pointer, the
 * bounds, the sizes and the view stay those of create.
 *   - visit_budget: the visit capacity of every frame (see
 *     vkhr_set_visit_budget); 0 counts this frame's visits once (a host read)
 *     and uses 1.25x that.  A frame above it reports VKHR_ERR_CAPACITY from
 *     vkhr_check_status.  The context keeps the budget.
 *   - Create makes one uncaptured frame (so every scratch buffer has its
 *     size) and synchronises `stream`; launch never allocates or syncs.
 *   - The graph reads the context's staged job table at every replay: while
 *     it is in use the context runs no other voxelization.
 *   - The graph holds the addresses of the context's scratch buffers: until
 *     it is destroyed, a call on the context that would have to grow a
 *     scratch buffer fails with VKHR_ERR_CAPACITY instead of moving it.
 *     Destroy the graph before its context.
 *   - No reference counterpart as an API (the reference re-records command
 *     buffers per frame). */
typedef struct vkhr_frame_graph vkhr_frame_graph;

vkhr_status vkhr_frame_graph_create(vkhr_ctx* ctx, int32_t segments, const vkhr_voxel_job* job, int32_t normalize,
                                    uint64_t visit_budget, const vkhr_raymarch_params* params, const float* d_depth_in,
                                    float* d_rgba, float* d_depth_out, void* stream, vkhr_frame_graph** out);
vkhr_status vkhr_frame_graph_launch(vkhr_frame_graph* graph, void* stream);
vkhr_status vkhr_frame_graph_destroy(vkhr_frame_graph* graph);

/* ---- .hair files and strand reduction ------------------------------------- */

/* The 128-byte header of a `.hair` file, byte for byte
 * (HairStyle::FileHeader, hair_style.hh:147-174; the field bit-field as one
 * little-endian word of VKHR_HAIR_* bits). */
typedef struct vkhr_hair_header {
    char signature[4]; /* 'H', 'A', 'I', 'R' */
    uint32_t strand_count, vertex_count;
    uint32_t fields;
    uint32_t default_segment_count;
    float default_thickness, default_transparency;
    float default_color[3];
    char information[64];
    float bounding_box_min[3], bounding_box_max[3];
} vkhr_hair_header;

#define VKHR_HAIR_SEGMENTS 1u
#define VKHR_HAIR_VERTICES 2u
#define VKHR_HAIR_THICKNESS 4u
#define VKHR_HAIR_TRANSPARENCY 8u
#define VKHR_HAIR_COLOR 16u
#define VKHR_HAIR_TANGENTS 32u
#define VKHR_HAIR_INDICES 64u
#define VKHR_HAIR_BOUNDING_BOX 128u

/* Reads a file's header (no CUDA call).  VKHR_ERR_INVALID_ARG when the file
 * cannot be opened or read, or its signature is not HAIR. */
vkhr_status vkhr_hair_read_header(const char* path, vkhr_hair_header* header);

/* HairStyle::load (hair_style.cc:24-45, field readers :576-623) into device
 * memory: the segment count of every strand to h_segments (host, strand_count
 * of them; may be NULL), the vertices (float3) to d_vertices, and, when the
 * file holds them, the tangents (float3) to d_tangents and the indices (u32,
 * 2 per segment, 2 * (vertex_count - strand_count)) to d_indices (each may
 * be NULL).  The arrays stream through two pinned chunks with asynchronous
 * copies on `stream`; the call returns once they are done.  Thickness,
 * transparency and colour are skipped (nothing on the path reads them).
 * Errors (VKHR_ERR_INVALID_ARG, with the reference's error name in
 * vkhr_last_error): OpeningFile, ReadingFileHeader, InvalidSignature,
 * Reading<Field> for a short file, InvalidFormat for a file without
 * vertices. */
vkhr_status vkhr_hair_load(vkhr_ctx* ctx, const char* path, vkhr_hair_header* header, uint16_t* h_segments,
                           float* d_vertices, float* d_tangents, uint32_t* d_indices, void* stream);

/* HairStyle::reduce(ratio) (hair_style.cc:375-449) on device-resident
 * strands.  The choice of strands is the reference's, made on the host over
 * h_segments (NULL: every strand has default_segment_count segments): its
 * xorshift64 sequence from *seed (updated), its FP32 count arithmetic (ratio
 * 1 keeps every strand, shuffled: HairStyle::shuffle).  A kernel then gathers
 * the kept strands' vertices and tangents (d_tangents may be NULL), in the
 * order kept, to the outputs (capacity: the input's vertex count).  The kept
 * strands' segment counts go to h_segments_out (capacity strand_count), the
 * kept counts to *strands_out / *vertices_out.  Returns once the gather is
 * done.  Indices: vkhr_generate_indices over the kept segments. */
vkhr_status vkhr_reduce_strands(vkhr_ctx* ctx, float ratio, uint64_t* seed, const uint16_t* h_segments,
                                uint32_t strand_count, uint32_t default_segment_count, const float* d_vertices,
                                const float* d_tangents, uint16_t* h_segments_out, uint32_t* strands_out,
                                uint32_t* vertices_out, float* d_vertices_out, float* d_tangents_out, void* stream);

/* ---- compositing: the PPLL resolve and its PPLL-free form ---------------------
 * Colour images are width*height RGBA8 words, red in the low byte: the
 * colour attachment resolve.comp reads as the background and overwrites
 * (share/shaders/transparency/resolve.comp:6, :39, :101).  Loads convert
 * c / 255; stores clamp to [0, 1] and take the nearest code, ties to even
 * (Vulkan's UNORM conversions, whose ties the specs leave open).  Blends are
 * mix(x, y, a) = x * (1 - a) + y * a in FP32 without contraction. */
#define VKHR_PPLL_NULL 0xffffffffu  /* PPLL_NULL_NODE, ppll.glsl:4 */
#define VKHR_K_BUFFER_SIZE 16       /* resolve.comp:12 */
#define VKHR_MAX_FRAGMENTS 1024     /* resolve.comp:13 */

/* Node of the reference's per-pixel linked list (ppll.glsl:7-11;
 * LinkedList::NodeSize, include/vkhr/rasterizer/linked_list.hh:29):
 * color = packUnorm4x8(rgba), depth unpacked, prev = next node of the list. */
typedef struct vkhr_ppll_node {
    uint32_t color;
    float depth;
    uint32_t prev;
} vkhr_ppll_node;

/* A fragment for the PPLL-free composite: a node whose link is replaced by
 * its pixel, y * width + x. */
typedef struct vkhr_fragment {
    uint32_t color;
    float depth;
    uint32_t pixel;
} vkhr_fragment;

/* Replaces LinkedList::resolve (src/vkhr/rasterizer/linked_list.cc:21-41)
 * and resolve.comp:15-101: every pixel whose head is not VKHR_PPLL_NULL
 * blends its list over d_color: the first 16 nodes fill a k-buffer, up to
 * 1024 more are blended as they come (each swapped with the k-buffer's
 * furthest node when nearer), then the k-buffer back to front.
 *   d_heads  width*height words;  d_nodes  node_count nodes.
 * A link outside [0, node_count) ends its list (the reference reads past
 * its buffer there); vkhr_check_status reports it as VKHR_ERR_INVALID_ARG.
 * Never waits on the host. */
vkhr_status vkhr_resolve_ppll(vkhr_ctx* ctx, const uint32_t* d_heads, const vkhr_ppll_node* d_nodes,
                              uint32_t node_count, int32_t width, int32_t height, uint32_t* d_color, void* stream);

/* The colour pass's transparency without a linked list (strand.frag:81-84,
 * volume.frag:97-100, resolve.comp:15-101).  Each pixel resolves exactly the
 * list a PPLL would hold had the strand fragments been linked in buffer order
 * and the volume fragment after them (the raymarch runs in the subpass after
 * the strands, src/vkhr/rasterizer.cc:245-257): the volume fragment first,
 * then the strand fragments last-in first.  The result equals
 * vkhr_resolve_ppll on that PPLL, without its node pool: no fragment is
 * dropped for capacity (the reference keeps at most 32 per pixel on average,
 * ppll.glsl:25, linked_list.hh:28).
 *   d_fragments     fragment_count strand fragments (device memory);
 *   d_volume_rgba,  vkhr_raymarch's outputs (width*height float4 and floats)
 *   d_volume_depth  or both NULL: a pixel holds a volume fragment where its
 *                   depth is below 1 (vkhr_raymarch writes 1 where none
 *                   survives), coloured packUnorm4x8(rgba);
 *   d_color         the background, overwritten where a pixel has fragments.
 * A fragment whose pixel is outside the image is skipped and reported by
 * vkhr_check_status (VKHR_ERR_INVALID_ARG).  Scratch: 12 bytes per fragment
 * and about 8 per pixel, grow-only in the context; the call never waits on
 * the host and can be captured into a CUDA graph after one uncaptured call
 * at the same sizes. */
vkhr_status vkhr_composite(vkhr_ctx* ctx, const vkhr_fragment* d_fragments, uint32_t fragment_count,
                           const float* d_volume_rgba, const float* d_volume_depth, int32_t width, int32_t height,
                           uint32_t* d_color, void* stream);

/* Level of detail on the host.  vkhr_level_of_detail is Rasterizer::update's
 * glm::smoothstep(magnified, minified, distance) (rasterizer.cc:165-167);
 * vkhr_lod is scheme.glsl:7-11's lod(), which scales the raymarch's coverage
 * by lod and the strands' by 1 - lod (volume.frag:48, strand.frag:42); the
 * two predicates are Interface::rasterizer_enabled / raymarcher_enabled
 * (src/vkhr/rasterizer/interface.cc:534-540), which decide whether the
 * strands and the volume are drawn at all. */
float vkhr_level_of_detail(float magnified_distance, float minified_distance, float distance);
float vkhr_lod(int32_t renderer, float magnified_distance, float minified_distance, float distance);
int32_t vkhr_rasterizer_enabled(int32_t renderer, float level_of_detail);
int32_t vkhr_raymarcher_enabled(int32_t renderer, float level_of_detail);

#ifdef __cplusplus
}
#endif

#endif /* VKHR_CUDA_H */
