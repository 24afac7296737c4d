// ref_raymarch.cc -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's fragment shader share/shaders/volumes/volume.frag
// (with every include: volume_rendering.glsl, sample_volume.glsl,
// local_ambient_occlusion.glsl, approximate_deep_shadows.glsl,
// kajiya-kay.glsl, scheme.glsl, ...) as C++ through glslshim/glsl.hpp and runs
// it once per covered pixel on the CPU.  The Makefile strips the `#version`
// line into _ref/volume_frag.glsl.inc; no other line of the shader changes.
//
// What stands in for the Vulkan pipeline around the shader:
//   * the uniform blocks (camera.glsl:4-11, lights.glsl:4-19, params.glsl:7-33,
//     strand.glsl:8-16) are declared below and filled from vkhr_raymarch_params;
//   * the rasterizer of the proxy cube is oracle_pixel_entry_inv (FP64);
//   * the PPLL append (ppll.glsl:23-48) records the fragment's colour/depth;
//   * packUnorm4x8's clamp to [0, 1] (ppll.glsl:32) is applied to the colour.
#include <cmath>
#include <cstdint>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "glsl.hpp"
#include "../vkhr_oracle.h"

#undef M_PI
#undef M_E

namespace glsl {

#define VKHR_CAMERA_GLSL
#define VKHR_LIGHTS_GLSL
#define VKHR_PARAMS_GLSL
#define VKHR_STRAND_GLSL
#define VKHR_PPLL_GLSL
#define YES 1
#define NO 0
#define PPLL_NULL_NODE 0xffffffffu

// camera.glsl:4-11
struct Camera {
    mat4 view;
    mat4 projection;
    vec3 position;
    float look_at_distance;
    float near, far;
    vec2 resolution;
};
static Camera camera;

// lights.glsl:4-19
struct Light {
    vec3 vector;
    float type;
    vec3 intensity;
    float cutoff;
    mat4 matrix;
    vec3 origin;
    float near;
    float far;
};
static Light lights[1];

// params.glsl:7-33
static int shading_model, deep_shadows_kernel_size, deep_shadows_sampling_type, deep_shadows_stride_size,
    deep_shadows_on, pcf_shadows_kernel_size, pcf_shadows_sampling_type;
static float pcf_shadows_bias;
static int pcf_shadows_on, shadow_technique;
static float isosurface, raycast_steps, occlusion_radius, ao_exponent, ao_max, magnified_distance;
static int renderer;
static float minified_distance;
static int benchmarking;

#include "bounding_box.glsl"

// strand.glsl:8-16
static AABB volume_bounds;
static vec3 volume_resolution;
static float strand_width;
static vec3 hair_color;
static float hair_alpha;
static float hair_exponent;
static float strand_ratio;

// Per-fragment state.
static thread_local vec4 gl_FragCoord;
static thread_local bool frag_emitted;
static thread_local vec4 frag_color;
static thread_local float frag_depth;
static thread_local float frag_subpass_depth;

static uint ppll_next_node() { return 0u; }
static void ppll_node_data(uint, vec4 c, float d) { frag_color = c; frag_depth = d; frag_emitted = true; }
static void ppll_link_node(ivec2, uint) {}
static vec4 glsl_subpass_load() { return vec4(frag_subpass_depth, 0.0f, 0.0f, 0.0f); }

#define layout(...) static thread_local
#define uniform
#define in struct
#define out
#define subpassLoad(x) glsl_subpass_load()
#define discard do { return; } while (0)
#define main ref_volume_frag_main
#include "volume_frag.glsl.inc"
#undef main
#undef discard
#undef subpassLoad
#undef out
#undef in
#undef uniform
#undef layout

static void set_mat(mat4& m, const float* f)
{
    for (int c = 0; c < 4; ++c) m.c[c] = vec4(f[4 * c + 0], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]);
}

static int tex_fmt_density(int f)
{
    return f == VKHR_DENSITY_U8_UNORM ? TEX_R8_UNORM : (f == VKHR_DENSITY_U32_COUNT ? TEX_R32_UINT_AS_FLOAT : TEX_R32F);
}

} // namespace glsl

// packUnorm4x8's clamp (ppll.glsl:32) with IEEE 754-2008 min/max: NaN -> 0.
static inline float clamp01(float x) { return x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f; }

// Runs volume.frag for rows [row_begin, row_end).  Only reference semantics:
// shadow_steps must be <= 0 (shadows use raycast_steps) and kd must be 1.
extern "C" int ref_raymarch(const vkhr_raymarch_params* p, const void* density, const void* tangent,
                            const float* depth_in, float* rgba, float* depth_out, int row_begin, int row_end,
                            int threads)
{
    using namespace glsl;
    if (p->shadow_steps > 0.0f || p->kd != 1.0f) return -1;
    set_mat(camera.view, p->view);
    set_mat(camera.projection, p->projection);
    camera.position = vec3(p->camera_position[0], p->camera_position[1], p->camera_position[2]);
    camera.look_at_distance = p->look_at_distance;
    camera.resolution = vec2((float)p->width, (float)p->height);
    lights[0].origin = vec3(p->light_origin[0], p->light_origin[1], p->light_origin[2]);
    lights[0].intensity = vec3(p->light_intensity[0], p->light_intensity[1], p->light_intensity[2]);
    shading_model = p->shading_model;
    deep_shadows_on = p->deep_shadows_on;
    isosurface = p->isosurface;
    raycast_steps = p->raycast_steps;
    occlusion_radius = p->occlusion_radius;
    ao_exponent = p->ao_exponent;
    ao_max = p->ao_max;
    magnified_distance = p->magnified_distance;
    renderer = p->renderer;
    minified_distance = p->minified_distance;
    for (int c = 0; c < 3; ++c) {
        volume_bounds.origin = vec3(p->volume_bounds.origin[0], p->volume_bounds.origin[1], p->volume_bounds.origin[2]);
        volume_bounds.size = vec3(p->volume_bounds.size[0], p->volume_bounds.size[1], p->volume_bounds.size[2]);
    }
    volume_bounds.radius = p->volume_bounds.radius;
    volume_bounds.volume = p->volume_bounds.volume;
    volume_resolution = vec3((float)p->volume_resolution[0], (float)p->volume_resolution[1], (float)p->volume_resolution[2]);
    hair_color = vec3(p->hair_color[0], p->hair_color[1], p->hair_color[2]);
    hair_alpha = p->hair_alpha;
    hair_exponent = p->hair_exponent;

    double inv[16];
    const int inv_ok = oracle_vp_inverse(p, inv);
    const int W = p->width;
    if (threads <= 0) threads = oracle_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int y = row_begin; y < row_end; ++y) {
        strand_density.data = density;
        strand_density.format = tex_fmt_density(p->density_format);
        strand_tangent.data = tangent;
        strand_tangent.format = p->tangent_format == VKHR_TANGENT_I8_SNORM ? TEX_RGBA8_SNORM : TEX_RGBA32F;
        for (int c = 0; c < 3; ++c) strand_density.n[c] = strand_tangent.n[c] = p->volume_resolution[c];
        for (int x = 0; x < W; ++x) {
            std::size_t at = (std::size_t)y * (std::size_t)W + (std::size_t)x;
            float* o = rgba + 4 * at;
            o[0] = o[1] = o[2] = o[3] = 0.0f;
            if (depth_out) depth_out[at] = 1.0f;
            double st[3];
            if (!inv_ok || !oracle_pixel_entry_inv(p, inv, x, y, st)) continue;
            fs_in.position = vec4((float)st[0], (float)st[1], (float)st[2], 1.0f);
            gl_FragCoord = vec4((float)x + 0.5f, (float)y + 0.5f, 0.0f, 1.0f);
            frag_subpass_depth = depth_in ? depth_in[at] : 1.0f;
            frag_emitted = false;
            ref_volume_frag_main();
            if (!frag_emitted) continue;
            o[0] = clamp01(frag_color.x);
            o[1] = clamp01(frag_color.y);
            o[2] = clamp01(frag_color.z);
            o[3] = clamp01(frag_color.w);
            if (depth_out) depth_out[at] = frag_depth;
        }
    }
    return 0;
}
