/*
 * vkhr_oracle.h -- CPU oracle for vkhr's volumetric level-of-detail path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms, used as the checker in tests/, in __graft_entry__.smoke() and as
 * the timed CPU baseline in bench.py.  No product code path links or calls it.
 *
 * Voxelizer: strict IEEE FP32 in the reference's operation order (build with
 * -O2 -fno-fast-math -ffp-contract=off); bit-exact with the reference's own
 * hair_style.cc compiled from its sources (oracle/_ref, see oracle/Makefile).
 * Raymarcher: a transcription of share/shaders/volumes/volume.frag and its
 * includes, instantiated in FP64 (the parity oracle; loop variables `t` stay
 * FP32 as in GLSL so iteration counts match) and in FP32 (CPU baseline).
 */
#ifndef VKHR_ORACLE_H
#define VKHR_ORACLE_H

#include <stdint.h>
#include <stddef.h>
#include "../include/vkhr_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* hair_style.cc:215-255 (generate_bounding_box + get_bounding_box). */
void oracle_bounding_box(const float* vertices, uint32_t vertex_count, vkhr_aabb* out);

/* hair_style.cc:171-194. tangents: vertex_count float3. */
void oracle_generate_tangents(const float* vertices, const uint16_t* segments, uint32_t strand_count,
                              float* tangents);

/* hair_style.cc:196-213. indices: 2*sum(segments) uint32. */
void oracle_generate_indices(const uint16_t* segments, uint32_t strand_count, uint32_t* indices);

/* hair_style.cc:257-294.  counts: uint32 (never saturating), densities: u8
 * (reference, saturating at 255), tangents_q: int8 x4 per voxel (w = 0).
 * Any output may be NULL.  Returns the number of dropped visits (coordinates
 * whose index falls outside the grid; undefined behaviour in the reference). */
uint64_t oracle_voxelize_vertices(const float* vertices, const float* tangents, uint32_t vertex_count,
                                  const vkhr_aabb* bounds, int w, int h, int d, int index_mode,
                                  uint32_t* counts, uint8_t* densities, int8_t* tangents_q);

/* hair_style.cc:296-342. */
uint64_t oracle_voxelize_segments(const float* vertices, const float* tangents, const uint32_t* indices,
                                  uint64_t index_count, const vkhr_aabb* bounds, int w, int h, int d,
                                  int index_mode, uint32_t* counts, uint8_t* densities, int8_t* tangents_q);

/* Number of voxels one segment visits (the reference's `while (steps-- > 0.0f)`). */
uint32_t oracle_segment_visits(const float* vertices, const uint32_t* indices, uint64_t pair,
                               const vkhr_aabb* bounds, int w, int h, int d);

/* hair_style.cc:344-357 (constant volume -> 0, the reference divides by 0). */
void oracle_normalize(uint8_t* densities, uint64_t n);
void oracle_downsample(const uint8_t* in, int w, int h, int d, int filter, uint8_t* out);

/* Texel format of the differentiable oracle: double densities, double x4
 * tangents (so that finite-difference perturbations are exact). */
#define ORACLE_F64 100

/* The differentiable raymarch in FP64 (adjoint.c): the loss
 * sum((rgba - target)^2) with rgba kept in double, over the pixels whose
 * mask byte is nonzero (mask NULL: all), and its analytic gradient
 * (accumulated into g_density, g_tangent (4 per voxel), g_params
 * [kd, hair_exponent]; any may be NULL).  density / tangent in ORACLE_F64. */
double oracle_diff_loss(const vkhr_raymarch_params* p, const double* density, const double* tangent,
                        const float* target, const uint8_t* mask, double* g_density, double* g_tangent,
                        double* g_params, int threads);
/* Trilinear splat of vertices in FP64 (accumulated into density) and its adjoint. */
void oracle_splat(const float* vertices, uint32_t n, const vkhr_aabb* b, int w, int h, int d, double* density);
void oracle_splat_adjoint(const float* vertices, uint32_t n, const vkhr_aabb* b, int w, int h, int d,
                          const double* g_density, double* g_vertices);

/* Rasterizer stand-in for the proxy cube (volume.vert:17-25, volume.cc:60-102,
 * back-face culling): world-space entry point of the ray through the centre
 * of pixel (px, py) into the AABB.  Returns 0 when no front face covers it. */
int oracle_pixel_entry(const vkhr_raymarch_params* p, int px, int py, double start[3]);
/* The same with inverse(projection * view) precomputed by oracle_vp_inverse. */
int oracle_vp_inverse(const vkhr_raymarch_params* p, double inv[16]);
int oracle_pixel_entry_inv(const vkhr_raymarch_params* p, const double inv[16], int px, int py, double start[3]);

/* Per-pixel diagnostics of the FP64 raymarch. */
typedef struct oracle_pixel_diag {
    double iso_margin;   /* min over nonzero samples of |acc - iso| / iso (inf if none) */
    double support_margin; /* min over samples taken before the surface froze of their
                              distance in texels to flipping `density != 0` (see
                              support_margin in raymarch_body.h; inf if none)          */
    double tangent_len;  /* length of the sampled tangent before normalisation         */
    double iso_shift;    /* min over nonzero samples k of |acc_k - iso| / sum_{i<=k} |grad rho_i|_1:
                            how far, in texels, every sample up to k would have to
                            move to flip that sample's isosurface test (inf if none)  */
    double fp32_res;     /* FP32 position resolution of the ray's samples, in texels:
                            2^-24 (|start| + radius) max_k N_k / size_k (the samples
                            mix(start, end, t) of an entry point and end point
                            that are exact up to their own rounding)           */
    int32_t steps_taken; /* primary-loop iterations executed                          */
    int32_t covered;     /* 1 if the pixel spawned a ray                              */
} oracle_pixel_diag;

/* volume.frag:31-103 over rows [row_begin, row_end) with `threads` OpenMP
 * threads (<= 0: all).  rgba: width*height*4, depth_out: width*height (may be
 * NULL), diag: width*height (may be NULL, FP64 only).  depth_in may be NULL. */
void oracle_raymarch_f64(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                         const float* depth_in, float* rgba, float* depth_out, oracle_pixel_diag* diag,
                         int row_begin, int row_end, int threads);
void oracle_raymarch_f32(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                         const float* depth_in, float* rgba, float* depth_out,
                         int row_begin, int row_end, int threads);

int oracle_max_threads(void);

/* ---- compositing (resolve.c) ---------------------------------------------
 * Colours are RGBA8 words, red in the low byte (packUnorm4x8's order). */

/* Vulkan's float -> UNORM8 conversion of 4 channels: clamp to [0, 1] (NaN to
 * 0), scale by 255, nearest code with ties to even. */
uint32_t oracle_pack_unorm8x4(const float v[4]);

/* resolve.comp:15-101 over the reference's PPLL: heads (width*height words,
 * 0xffffffff = empty), nodes of 3 words {color, depth bits, prev}.  color is
 * read as the background and written where a list is non-empty.  Returns 0,
 * or -1 when a list links a node index >= node_count (that list ends there). */
int oracle_resolve_ppll(const uint32_t* heads, const uint32_t* nodes, uint32_t node_count, int width, int height,
                        uint32_t* color, int threads);

/* The PPLL-free composite: fragments of 3 words {color, depth bits, pixel};
 * a pixel holds a volume fragment where volume_depth < 1 (volume_rgba /
 * volume_depth may be NULL).  Each pixel resolves the list a PPLL holds after
 * the fragments were linked in buffer order and the volume fragment last.
 * Returns 0, or -1 (nothing written) when a pixel index is out of range. */
int oracle_composite(const uint32_t* fragments, uint32_t fragment_count, const float* volume_rgba,
                     const float* volume_depth, int width, int height, uint32_t* color, int threads);

#ifdef __cplusplus
}
#endif

#endif
