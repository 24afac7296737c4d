// ref_hair.cc -- TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own vkhr::HairStyle::load / save /
// reduce (src/vkhr/scene_graph/hair_style.cc, compiled unmodified into
// _ref), so that tests can pin the `.hair` and reduction restatements to the
// reference code.  HairStyle keeps its random seed private (it seeds it from
// std::random_device); this wrapper alone sees the class's members as public,
// so that a test can fix the seed and read it back.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include <glm/glm.hpp>

#define private public
#include <vkhr/scene_graph/hair_style.hh>
#undef private

namespace {

void fill_vec3(std::vector<glm::vec3>& out, const float* f, std::size_t n)
{
    out.resize(n);
    for (std::size_t i = 0; i < n; ++i) out[i] = glm::vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
}

void copy_vec3(const std::vector<glm::vec3>& in, float* f)
{
    for (std::size_t i = 0; i < in.size(); ++i) {
        f[3 * i] = in[i].x;
        f[3 * i + 1] = in[i].y;
        f[3 * i + 2] = in[i].z;
    }
}

} // namespace

// HairStyle::load: the error state (0 = none), the counts, the field bits
// and, where the buffers are given and large enough, the arrays.
extern "C" int ref_hair_load(const char* path, uint32_t* strands, uint32_t* verts, uint32_t* fields, uint32_t* index_count,
                             uint16_t* segments, uint32_t cap_strands, float* vertices, float* tangents,
                             uint32_t cap_verts, uint32_t* indices, uint32_t cap_indices)
{
    vkhr::HairStyle h{};
    h.load(path);
    const int err = (int)h.get_last_error_state();
    *strands = (uint32_t)h.segments.size();
    *verts = (uint32_t)h.vertices.size();
    *index_count = (uint32_t)h.indices.size();
    uint32_t bits = 0;
    std::memcpy(&bits, &h.file_header.field, sizeof(bits));
    *fields = bits;
    if (segments && h.segments.size() <= cap_strands)
        std::memcpy(segments, h.segments.data(), h.segments.size() * sizeof(uint16_t));
    if (vertices && h.vertices.size() <= cap_verts) copy_vec3(h.vertices, vertices);
    if (tangents && h.tangents.size() <= cap_verts) copy_vec3(h.tangents, tangents);
    if (indices && h.indices.size() <= cap_indices)
        std::memcpy(indices, h.indices.data(), h.indices.size() * sizeof(uint32_t));
    return err;
}

// HairStyle::save of the given arrays (tangents may be NULL).
extern "C" int ref_hair_save(const char* path, const uint16_t* segments, uint32_t strand_count, const float* vertices,
                             const float* tangents, uint32_t vertex_count)
{
    vkhr::HairStyle h{};
    h.segments.assign(segments, segments + strand_count);
    fill_vec3(h.vertices, vertices, vertex_count);
    if (tangents) fill_vec3(h.tangents, tangents, vertex_count);
    return h.save(path) ? 0 : (int)h.get_last_error_state() + 1000;
}

// HairStyle::reduce(ratio) with the seed fixed: the kept vertices and
// tangents (capacity: vertex_count each), the kept segment counts (capacity:
// strand_count), the kept counts and the seed after.  segments may be NULL
// (every strand then has default_segment_count segments).
extern "C" void ref_reduce(const float* vertices, const float* tangents, uint32_t vertex_count, const uint16_t* segments,
                           uint32_t strand_count, uint32_t default_segment_count, float ratio, uint64_t* seed,
                           float* vertices_out, float* tangents_out, uint16_t* segments_out, uint32_t* strands_kept,
                           uint32_t* vertices_kept)
{
    vkhr::HairStyle h{};
    fill_vec3(h.vertices, vertices, vertex_count);
    if (tangents) fill_vec3(h.tangents, tangents, vertex_count);
    if (segments) h.segments.assign(segments, segments + strand_count);
    else h.file_header.strand_count = strand_count;
    h.file_header.default_segment_count = default_segment_count;
    h.seed = *seed;
    h.reduce(ratio);
    *seed = h.seed;
    *strands_kept = (uint32_t)h.segments.size();
    *vertices_kept = (uint32_t)h.vertices.size();
    copy_vec3(h.vertices, vertices_out);
    if (tangents) copy_vec3(h.tangents, tangents_out);
    std::memcpy(segments_out, h.segments.data(), h.segments.size() * sizeof(uint16_t));
}
