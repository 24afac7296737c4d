// facade_test.cc -- drives the C++ facade (include/vkhr/cuda.hh) the way the
// reference's host would: a HairStyle-shaped object with std::vector members
// is voxelized (both modes), normalized and raymarched; outputs are written
// as raw files for tests/test_gpu_cxx_facade.py to compare with the oracle.
//
//   facade_test <in.bin> <out_prefix>
// in.bin: uint32 nv, uint32 nidx, int32 res[3], float aabb[8], float vertices[3nv],
//         float tangents[3nv], uint32 indices[nidx], vkhr_raymarch_params
#include <vkhr/cuda.hh>

#include <cstdio>
#include <fstream>
#include <iostream>

struct vec3 {
    float x, y, z;
};
struct AABB {
    float origin[3];
    float radius;
    float size[3];
    float volume;
};
struct Style {  // the members of vkhr::HairStyle the voxelizer reads
    std::vector<vec3> vertices, tangents;
    std::vector<unsigned> indices;
    AABB aabb;
    AABB get_bounding_box() const { return aabb; }
};

template <class T>
static void write(const std::string& path, const std::vector<T>& v)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    uint32_t nv = 0, nidx = 0;
    int32_t res[3];
    Style s;
    in.read(reinterpret_cast<char*>(&nv), 4);
    in.read(reinterpret_cast<char*>(&nidx), 4);
    in.read(reinterpret_cast<char*>(res), 12);
    in.read(reinterpret_cast<char*>(&s.aabb), 32);
    s.vertices.resize(nv);
    s.tangents.resize(nv);
    s.indices.resize(nidx);
    in.read(reinterpret_cast<char*>(s.vertices.data()), 12 * nv);
    in.read(reinterpret_cast<char*>(s.tangents.data()), 12 * nv);
    in.read(reinterpret_cast<char*>(s.indices.data()), 4 * nidx);
    vkhr_raymarch_params p;
    in.read(reinterpret_cast<char*>(&p), sizeof(p));
    // compositing inputs: strand fragments, the background, a PPLL
    const size_t px = (size_t)p.width * (size_t)p.height;
    uint32_t nf = 0, nn = 0;
    in.read(reinterpret_cast<char*>(&nf), 4);
    std::vector<vkhr_fragment> frags(nf);
    in.read(reinterpret_cast<char*>(frags.data()), 12 * (size_t)nf);
    std::vector<uint32_t> background(px), heads(px);
    in.read(reinterpret_cast<char*>(background.data()), 4 * px);
    in.read(reinterpret_cast<char*>(&nn), 4);
    std::vector<vkhr_ppll_node> nodes(nn);
    in.read(reinterpret_cast<char*>(heads.data()), 4 * px);
    in.read(reinterpret_cast<char*>(nodes.data()), 12 * (size_t)nn);
    if (!in) return 3;
    try {
        vkhr::cuda::Context ctx(0);
        vkhr::cuda::Volume vv = vkhr::cuda::voxelize_vertices(ctx, s, res[0], res[1], res[2]);
        vkhr::cuda::Volume vs = vkhr::cuda::voxelize_segments(ctx, s, res[0], res[1], res[2]);
        write(std::string(argv[2]) + "_v_dens.bin", vv.densities);
        write(std::string(argv[2]) + "_v_tan.bin", vv.tangents);
        write(std::string(argv[2]) + "_s_dens.bin", vs.densities);
        write(std::string(argv[2]) + "_s_tan.bin", vs.tangents);
        write(std::string(argv[2]) + "_s_counts.bin", vs.counts);
        vs.normalize(ctx);
        write(std::string(argv[2]) + "_s_norm.bin", vs.densities);
        vkhr::Raymarcher rm(ctx);
        vkhr::Raymarcher::Image img = rm.draw(vs, p);
        write(std::string(argv[2]) + "_rgba.bin", img.rgba);
        write(std::string(argv[2]) + "_depth.bin", img.depth);
        // the colour pass's resolve: over the reference's lists, and without them
        vkhr::LinkedList ll(ctx, (uint32_t)p.width, (uint32_t)p.height);
        write(std::string(argv[2]) + "_ppll.bin", ll.resolve(heads, nodes, background));
        write(std::string(argv[2]) + "_composite.bin", ll.composite(frags, background, &img));
        try {
            ll.composite(frags, std::vector<uint32_t>(px + 1));
            return 6;
        } catch (const vkhr::cuda::Error& e) {
            if (e.status != VKHR_ERR_INVALID_ARG) return 7;
        }
        // errors surface as exceptions with the ABI status
        try {
            vkhr::cuda::voxelize_vertices(ctx, s, 0, res[1], res[2]);
            return 4;
        } catch (const vkhr::cuda::Error& e) {
            if (e.status != VKHR_ERR_INVALID_ARG) return 5;
        }
    } catch (const std::exception& e) {
        std::cerr << "facade_test: " << e.what() << "\n";
        return 1;
    }
    std::cout << "facade ok\n";
    return 0;
}
