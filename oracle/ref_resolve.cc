// ref_resolve.cc -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's compute shader share/shaders/transparency/
// resolve.comp, with its include ppll.glsl, as C++ through glslshim/glsl.hpp
// and runs it once per pixel on the CPU.  The Makefile strips the `#version`
// line into _ref/resolve_comp.glsl.inc; no other line of the shader changes.
//
// What stands in for the Vulkan objects around the shader:
//   * the storage image of heads (binding 5), the node buffer (6), its size
//     (7) and counter (8) of ppll.glsl, and the colour image (9) of
//     resolve.comp are the globals the shader's declarations become below;
//   * the dispatch of ceil(w/8) x ceil(h/8) groups of 8x8 (linked_list.cc:40)
//     is a loop over the image's pixels (invocations outside it would only
//     reach imageLoad / imageStore outside the image);
//   * ref_build_ppll appends fragments with ppll.glsl's own ppll_next_node /
//     ppll_node_data / ppll_link_node, as strand.frag:81-84 and
//     volume.frag:97-100 call them, after the clear of LinkedList::clear
//     (heads to 0xffffffff, counter to 0).
#include <cstdint>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "glsl.hpp"
#include "../vkhr_oracle.h"

namespace glsl {

static thread_local uvec3 gl_GlobalInvocationID;

#define layout(...)
#define uniform
#define in
#define buffer static union
#define LinkedList
#define LinkedListCounter
#define Config static union
#define ppll_nodes (*ppll_nodes_ptr)
#define main ref_resolve_main
#include "resolve_comp.glsl.inc"
#undef main
#undef ppll_nodes
#undef Config
#undef LinkedListCounter
#undef LinkedList
#undef buffer
#undef in
#undef uniform
#undef layout

static_assert(sizeof(Node) == 12, "ppll.glsl's Node is 12 bytes");

} // namespace glsl

// resolve.comp over every pixel: heads (width*height words), nodes (node_count
// 12-byte nodes), color (width*height RGBA8 words, read and written).
extern "C" int ref_resolve_ppll(const uint32_t* heads, const void* nodes, uint32_t node_count, int width, int height,
                                uint32_t* color_words, int threads)
{
    using namespace glsl;
    (void)node_count;
    ppll_heads.data = const_cast<uint32_t*>(heads);
    ppll_heads.width = width;
    ppll_heads.height = height;
    ppll_nodes_ptr = (Node(*)[])const_cast<void*>(nodes);
    color.data = color_words;
    color.width = width;
    color.height = height;
    if (threads <= 0) threads = oracle_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
            ref_resolve_main();
        }
    return 0;
}

// Clears a PPLL of `capacity` nodes (the nodes buffer holds capacity + 1:
// ppll_next_node hands out index ppll_size too), then links the fragments
// (3 words {color, depth bits, pixel}) in buffer order and, when given, the
// volume fragment of every pixel whose volume_depth is below 1.  Returns the
// node counter after the appends.
extern "C" uint32_t ref_build_ppll(const uint32_t* fragments, uint32_t fragment_count, const float* volume_rgba,
                                   const float* volume_depth, int width, int height, uint32_t capacity,
                                   uint32_t* heads, void* nodes)
{
    using namespace glsl;
    const std::size_t npix = (std::size_t)width * (std::size_t)height;
    for (std::size_t p = 0; p < npix; ++p) heads[p] = 0xffffffffu;
    ppll_heads.data = heads;
    ppll_heads.width = width;
    ppll_heads.height = height;
    ppll_nodes_ptr = (Node(*)[])nodes;
    ppll_size = capacity;
    ppll_counter = 0;
    for (uint32_t i = 0; i < fragment_count; ++i) {
        const uint32_t* f = fragments + 3 * (std::size_t)i;
        float depth;
        std::memcpy(&depth, f + 1, 4);
        const ivec2 pixel((int)(f[2] % (uint32_t)width), (int)(f[2] / (uint32_t)width));
        uint node = ppll_next_node();
        if (node == PPLL_NULL_NODE) continue;
        ppll_node_data(node, unpackUnorm4x8(f[0]), depth);
        ppll_link_node(pixel, node);
    }
    if (volume_rgba && volume_depth)
        for (std::size_t p = 0; p < npix; ++p) {
            if (!(volume_depth[p] < 1.0f)) continue;
            const float* c = volume_rgba + 4 * p;
            const ivec2 pixel((int)(p % (std::size_t)width), (int)(p / (std::size_t)width));
            uint node = ppll_next_node();
            if (node == PPLL_NULL_NODE) continue;
            ppll_node_data(node, vec4(c[0], c[1], c[2], c[3]), volume_depth[p]);
            ppll_link_node(pixel, node);
        }
    return ppll_counter;
}
