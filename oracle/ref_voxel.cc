// ref_voxel.cc -- TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own vkhr::HairStyle (compiled from
// src/vkhr/scene_graph/hair_style.cc against glmshim/), so that tests can
// compare the C oracle with the reference code on the same inputs.
#include <vkhr/scene_graph/hair_style.hh>

#include <array>
#include <cstdint>
#include <cstring>

#include "vkhr_oracle.h"

static void fill_vec3(std::vector<glm::vec3>& out, const float* f, std::size_t n)
{
    out.resize(n);
    for (std::size_t i = 0; i < n; ++i) out[i] = glm::vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
}

// HairStyle::generate_tangents / generate_indices / generate_bounding_box.
extern "C" void ref_prepare(const float* vertices, uint32_t vertex_count, const uint16_t* segments,
                            uint32_t strand_count, float* tangents_out, uint32_t* indices_out, vkhr_aabb* aabb_out)
{
    vkhr::HairStyle h{};
    h.segments.assign(segments, segments + strand_count);
    fill_vec3(h.vertices, vertices, vertex_count);
    h.generate_tangents();
    h.generate_indices();
    h.generate_bounding_box();
    for (std::size_t i = 0; i < h.tangents.size(); ++i) {
        tangents_out[3 * i + 0] = h.tangents[i].x;
        tangents_out[3 * i + 1] = h.tangents[i].y;
        tangents_out[3 * i + 2] = h.tangents[i].z;
    }
    std::memcpy(indices_out, h.indices.data(), h.indices.size() * sizeof(unsigned));
    vkhr::AABB b = h.get_bounding_box();
    for (int c = 0; c < 3; ++c) {
        aabb_out->origin[c] = b.origin[c];
        aabb_out->size[c] = b.size[c];
    }
    aabb_out->radius = b.radius;
    aabb_out->volume = b.volume;
}

// HairStyle::voxelize_vertices (segments_mode = 0) or voxelize_segments (1)
// over the AABB of the vertices (generate_bounding_box), then optionally
// Volume::normalize.
extern "C" void ref_voxelize(int segments_mode, const float* vertices, uint32_t vertex_count, const float* tangents,
                             const uint32_t* indices, uint64_t index_count, int w, int h, int d, int normalize,
                             uint8_t* densities_out, int8_t* tangents_out)
{
    vkhr::HairStyle s{};
    fill_vec3(s.vertices, vertices, vertex_count);
    fill_vec3(s.tangents, tangents, vertex_count);
    s.indices.assign(indices, indices + index_count);
    s.generate_bounding_box();
    vkhr::HairStyle::Volume v = segments_mode ? s.voxelize_segments(w, h, d) : s.voxelize_vertices(w, h, d);
    if (normalize) v.normalize();
    std::memcpy(densities_out, v.densities.data(), v.densities.size());
    for (std::size_t i = 0; i < v.tangents.size(); ++i) {
        tangents_out[4 * i + 0] = v.tangents[i].x;
        tangents_out[4 * i + 1] = v.tangents[i].y;
        tangents_out[4 * i + 2] = v.tangents[i].z;
        tangents_out[4 * i + 3] = v.tangents[i].w;
    }
}

// Volume::downsample with the filters the ABI offers (0 max, 1 min, 2 floor
// of the mean, 3 saturating sum); the reference itself has no call site.
extern "C" void ref_downsample(const uint8_t* in, int w, int h, int d, int filter, uint8_t* out)
{
    vkhr::HairStyle::Volume v{glm::vec3(w, h, d), vkhr::AABB{}};
    v.densities.assign(in, in + (std::size_t)w * h * d);
    auto run = [&](auto f) {
        vkhr::HairStyle::Volume r = v.downsample(f);
        std::memcpy(out, r.densities.data(), r.densities.size());
    };
    if (filter == 0)
        run([](const std::array<unsigned char, 8>& n) { unsigned char m = 0; for (auto x : n) m = x > m ? x : m; return m; });
    else if (filter == 1)
        run([](const std::array<unsigned char, 8>& n) { unsigned char m = 255; for (auto x : n) m = x < m ? x : m; return m; });
    else if (filter == 2)
        run([](const std::array<unsigned char, 8>& n) { unsigned s = 0; for (auto x : n) s += x; return (unsigned char)(s / 8u); });
    else
        run([](const std::array<unsigned char, 8>& n) { unsigned s = 0; for (auto x : n) s += x; return (unsigned char)(s < 255u ? s : 255u); });
}
