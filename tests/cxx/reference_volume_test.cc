// The facade (include/vkhr/cuda.hh) against the reference's own
// include/vkhr/scene_graph/hair_style.hh (glm through oracle/glmshim):
//   * vkhr::cuda::voxelize_segments / voxelize_vertices instantiate for the
//     reference's vkhr::HairStyle (compiled, not run: that needs a GPU);
//   * vkhr::cuda::to_reference gives the reference's HairStyle::Volume, field
//     for field (run on the host).
#include <vkhr/scene_graph/hair_style.hh>

#include <vkhr/cuda.hh>

#include <cstdio>

#ifndef VKHR_CONVERSION_ONLY
vkhr::cuda::Volume facade_segments(vkhr::cuda::Context& ctx, const vkhr::HairStyle& style)
{
    return vkhr::cuda::voxelize_segments(ctx, style, 256, 256, 256);
}

vkhr::cuda::Volume facade_vertices(vkhr::cuda::Context& ctx, const vkhr::HairStyle& style)
{
    return vkhr::cuda::voxelize_vertices(ctx, style, 64, 64, 64);
}

// the loader's call site, src/vkhr/rasterizer/hair_style.cc:75, with the facade
vkhr::HairStyle::Volume loader_call_site(vkhr::cuda::Context& ctx, const vkhr::HairStyle& hair_style)
{
    auto strand_volume = vkhr::cuda::to_reference<vkhr::HairStyle::Volume>(
        vkhr::cuda::voxelize_segments(ctx, hair_style, 256, 256, 256));
    return strand_volume;
}
#endif

int main()
{
    vkhr::cuda::Volume v;
    v.resolution[0] = 3;
    v.resolution[1] = 2;
    v.resolution[2] = 4;
    const float origin[3] = {-1.5f, 0.25f, 2.0f}, size[3] = {3.0f, 1.0f, 0.5f};
    for (int k = 0; k < 3; ++k) {
        v.bounds.origin[k] = origin[k];
        v.bounds.size[k] = size[k];
    }
    v.bounds.radius = 3.2f;
    v.bounds.volume = 1.5f;
    const int n = 3 * 2 * 4;
    for (int i = 0; i < n; ++i) {
        v.densities.push_back((unsigned char)(i * 11));
        for (int c = 0; c < 4; ++c) v.tangents.push_back((int8_t)(c == 3 ? 0 : (i * 7 + c * 40) % 255 - 127));
    }
    const vkhr::HairStyle::Volume r = vkhr::cuda::to_reference<vkhr::HairStyle::Volume>(v);
    int bad = 0;
    bad += r.resolution.x != 3.0f || r.resolution.y != 2.0f || r.resolution.z != 4.0f;
    for (int k = 0; k < 3; ++k) bad += r.bounds.origin[k] != origin[k] || r.bounds.size[k] != size[k];
    bad += r.bounds.radius != 3.2f || r.bounds.volume != 1.5f;
    bad += (int)r.densities.size() != n || (int)r.tangents.size() != n;
    for (int i = 0; i < n && !bad; ++i) {
        bad += r.densities[i] != v.densities[i];
        bad += r.tangents[i].x != v.tangents[4 * i] || r.tangents[i].y != v.tangents[4 * i + 1] ||
               r.tangents[i].z != v.tangents[4 * i + 2] || r.tangents[i].w != v.tangents[4 * i + 3];
    }
    std::printf("%s\n", bad ? "mismatch" : "ok");
    return bad ? 1 : 0;
}
