// vkhr/cuda.hh -- C++17 facade over the C ABI (vkhr_cuda.h) for the vkhr host.
//
// Header-only; needs no CUDA headers: device memory goes through the ABI's
// vkhr_malloc / vkhr_upload / vkhr_download.  Errors from the ABI become
// vkhr::cuda::Error exceptions (the reference's Vulkan layer throws
// vkpp::Exception the same way, include/vkpp/exception.hh).
//
// Drop-in points in the reference:
//   * vkhr::cuda::voxelize_segments(style, 256, 256, 256) replaces
//     style.voxelize_segments(256, 256, 256) at src/vkhr/rasterizer/hair_style.cc:75
//     and returns the same HairStyle::Volume-shaped result (u8 densities,
//     i8vec4 tangents, resolution, bounds), bit-identical to it;
//   * vkhr::cuda::voxelize_vertices likewise for HairStyle::voxelize_vertices
//     (src/vkhr/scene_graph/hair_style.cc:257-294);
//   * vkhr::Raymarcher::draw renders the volume.frag raymarch
//     (share/shaders/volumes/volume.frag:31-103) headlessly into RGBA + depth;
//   * vkhr::LinkedList::resolve replaces vulkan::LinkedList::resolve
//     (src/vkhr/rasterizer/linked_list.cc:21-41, share/shaders/transparency/
//     resolve.comp:15-101) over the same per-pixel linked lists, and
//     LinkedList::composite resolves fragments without building the lists.
// The templates accept the reference's own vkhr::HairStyle (any type with
// `vertices`, `tangents`, `indices` vectors of 12-byte vec3 / uint32 and a
// get_bounding_box() returning an AABB-shaped struct).
#ifndef VKHR_CUDA_HH
#define VKHR_CUDA_HH

#include "../vkhr_cuda.h"

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace vkhr {
namespace cuda {

class Error : public std::runtime_error {
public:
    Error(vkhr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    vkhr_status status;
};

class Context {
public:
    explicit Context(int device = 0)
    {
        vkhr_status s = vkhr_create(device, &ctx_);
        if (s != VKHR_OK) throw Error(s, std::string("vkhr_create: ") + vkhr_status_string(s));
    }
    ~Context() { vkhr_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    vkhr_ctx* get() const { return ctx_; }

    void check(vkhr_status s) const
    {
        if (s != VKHR_OK) throw Error(s, vkhr_last_error(ctx_));
    }

    // ---- device buffers -----------------------------------------------------
    class Buffer {
    public:
        Buffer() = default;
        Buffer(const Context& c, size_t bytes) : ctx_(&c), bytes_(bytes) { c.check(vkhr_malloc(c.get(), bytes, &ptr_)); }
        ~Buffer() { release(); }
        Buffer(Buffer&& o) noexcept { *this = std::move(o); }
        Buffer& operator=(Buffer&& o) noexcept
        {
            if (this != &o) {
                release();
                ctx_ = o.ctx_;
                ptr_ = o.ptr_;
                bytes_ = o.bytes_;
                o.ptr_ = nullptr;
            }
            return *this;
        }
        void* data() const { return ptr_; }
        size_t size() const { return bytes_; }
        void upload(const void* src, size_t bytes, void* stream = nullptr) const
        {
            ctx_->check(vkhr_upload(ctx_->get(), ptr_, src, bytes, stream));
        }
        void download(void* dst, size_t bytes, void* stream = nullptr) const
        {
            ctx_->check(vkhr_download(ctx_->get(), dst, ptr_, bytes, stream));
        }

    private:
        void release()
        {
            if (ptr_ && ctx_) vkhr_free(ctx_->get(), ptr_);
            ptr_ = nullptr;
        }
        const Context* ctx_ = nullptr;
        void* ptr_ = nullptr;
        size_t bytes_ = 0;
    };

    template <class T>
    Buffer upload(const std::vector<T>& v, void* stream = nullptr) const
    {
        Buffer b(*this, v.size() * sizeof(T));
        b.upload(v.data(), v.size() * sizeof(T), stream);
        return b;
    }

    void sync(void* stream = nullptr) const { check(vkhr_sync(ctx_, stream)); }

private:
    vkhr_ctx* ctx_ = nullptr;
};

// HairStyle::Volume with the same fields as the reference (hair_style.hh:89-101)
// plus the exact uint32 counts.  `tangents` holds 4 int8 per voxel (i8vec4).
struct Volume {
    int resolution[3];
    vkhr_aabb bounds;
    std::vector<unsigned char> densities;
    std::vector<int8_t> tangents;  // x, y, z, w per voxel
    std::vector<uint32_t> counts;

    // Volume::normalize (hair_style.cc:344-357), on the host data.
    void normalize(Context& ctx)
    {
        Context::Buffer d(ctx, densities.size());
        d.upload(densities.data(), densities.size());
        ctx.check(vkhr_normalize_densities(ctx.get(), static_cast<uint8_t*>(d.data()), densities.size(), nullptr));
        d.download(densities.data(), densities.size());
        ctx.sync();
    }
};

template <class AABBLike>
vkhr_aabb to_aabb(const AABBLike& a)
{
    vkhr_aabb b;
    for (int c = 0; c < 3; ++c) {
        b.origin[c] = a.origin[c];
        b.size[c] = a.size[c];
    }
    b.radius = a.radius;
    b.volume = a.volume;
    return b;
}

namespace detail {
template <class Style>
Volume voxelize(Context& ctx, const Style& style, bool segments, int w, int h, int d, int index_mode)
{
    static_assert(sizeof(style.vertices[0]) == 12, "vertices must be 12-byte vec3");
    static_assert(sizeof(style.tangents[0]) == 12, "tangents must be 12-byte vec3");
    const size_t n = (size_t)w * (size_t)h * (size_t)d;
    Volume vol;
    vol.resolution[0] = w;
    vol.resolution[1] = h;
    vol.resolution[2] = d;
    vol.bounds = to_aabb(style.get_bounding_box());
    Context::Buffer v = ctx.upload(style.vertices);
    Context::Buffer t = ctx.upload(style.tangents);
    Context::Buffer counts(ctx, n * 4), dens(ctx, n), tq(ctx, n * 4);
    Context::Buffer idx;
    if (segments) idx = ctx.upload(style.indices);
    for (int attempt = 0;; ++attempt) {
        if (segments)
            ctx.check(vkhr_voxelize_segments(
                ctx.get(), static_cast<const float*>(v.data()), static_cast<const float*>(t.data()),
                static_cast<const uint32_t*>(idx.data()), style.indices.size(), &vol.bounds, w, h, d, index_mode,
                static_cast<uint32_t*>(counts.data()), static_cast<uint8_t*>(dens.data()),
                static_cast<int8_t*>(tq.data()), nullptr));
        else
            ctx.check(vkhr_voxelize_vertices(ctx.get(), static_cast<const float*>(v.data()),
                                             static_cast<const float*>(t.data()), (uint32_t)style.vertices.size(),
                                             &vol.bounds, w, h, d, index_mode, static_cast<uint32_t*>(counts.data()),
                                             static_cast<uint8_t*>(dens.data()), static_cast<int8_t*>(tq.data()),
                                             nullptr));
        // waits, and reports what the kernels recorded: a visit list sized
        // from an earlier call at this size that proved too small makes the
        // context count again, which the one retry does
        const vkhr_status s = vkhr_check_status(ctx.get(), nullptr);
        if (s == VKHR_ERR_CAPACITY && attempt == 0) continue;
        ctx.check(s);
        break;
    }
    vol.densities.resize(n);
    vol.tangents.resize(4 * n);
    vol.counts.resize(n);
    dens.download(vol.densities.data(), n);
    tq.download(vol.tangents.data(), 4 * n);
    counts.download(vol.counts.data(), 4 * n);
    ctx.sync();
    return vol;
}
} // namespace detail

// The reference's own HairStyle::Volume (include/vkhr/scene_graph/hair_style.hh:89-101:
// glm::vec3 resolution, AABB bounds, std::vector<unsigned char> densities,
// std::vector<glm::i8vec4> tangents) from a Volume, so that the loader's call
// site (src/vkhr/rasterizer/hair_style.cc:75) changes in one line:
//   auto strand_volume = vkhr::cuda::to_reference<vkhr::HairStyle::Volume>(
//       vkhr::cuda::voxelize_segments(ctx, hair_style, 256, 256, 256));
template <class RefVolume>
RefVolume to_reference(const Volume& v)
{
    RefVolume r;
    r.resolution = decltype(r.resolution)((float)v.resolution[0], (float)v.resolution[1], (float)v.resolution[2]);
    r.bounds.origin = decltype(r.bounds.origin)(v.bounds.origin[0], v.bounds.origin[1], v.bounds.origin[2]);
    r.bounds.radius = v.bounds.radius;
    r.bounds.size = decltype(r.bounds.size)(v.bounds.size[0], v.bounds.size[1], v.bounds.size[2]);
    r.bounds.volume = v.bounds.volume;
    r.densities.assign(v.densities.begin(), v.densities.end());
    typedef typename decltype(r.tangents)::value_type Tangent;
    const size_t n = v.tangents.size() / 4;
    r.tangents.reserve(n);
    for (size_t i = 0; i < n; ++i)
        r.tangents.push_back(Tangent(v.tangents[4 * i], v.tangents[4 * i + 1], v.tangents[4 * i + 2], v.tangents[4 * i + 3]));
    return r;
}

// HairStyle::voxelize_vertices (hair_style.cc:257-294) on the GPU.
template <class Style>
Volume voxelize_vertices(Context& ctx, const Style& style, int w, int h, int d,
                         int index_mode = VKHR_INDEX_REF_FP32)
{
    return detail::voxelize(ctx, style, false, w, h, d, index_mode);
}

// HairStyle::voxelize_segments (hair_style.cc:296-342) on the GPU.
template <class Style>
Volume voxelize_segments(Context& ctx, const Style& style, int w, int h, int d,
                         int index_mode = VKHR_INDEX_REF_FP32)
{
    return detail::voxelize(ctx, style, true, w, h, d, index_mode);
}

} // namespace cuda

// Headless raymarcher: the draw of vulkan::Volume (src/vkhr/rasterizer/volume.cc:104-112)
// with volume.frag, into device buffers; `Image` holds the host copy.
class Raymarcher {
public:
    struct Image {
        int width = 0, height = 0;
        std::vector<float> rgba;   // width*height*4, packUnorm4x8-clamped colour + coverage
        std::vector<float> depth;  // width*height, 1.0 where no fragment
    };

    explicit Raymarcher(cuda::Context& ctx) : ctx_(ctx) {}

    // Raymarch a normalized Volume (u8 densities, i8vec4 tangents) with the
    // UBO contents in `params` (density/tangent formats are set here).
    Image draw(const cuda::Volume& vol, vkhr_raymarch_params params)
    {
        params.density_format = VKHR_DENSITY_U8_UNORM;
        params.tangent_format = VKHR_TANGENT_I8_SNORM;
        for (int c = 0; c < 3; ++c) params.volume_resolution[c] = vol.resolution[c];
        params.volume_bounds = vol.bounds;
        cuda::Context::Buffer d = ctx_.upload(vol.densities);
        cuda::Context::Buffer t = ctx_.upload(vol.tangents);
        const size_t px = (size_t)params.width * (size_t)params.height;
        cuda::Context::Buffer rgba(ctx_, px * 16), depth(ctx_, px * 4);
        ctx_.check(vkhr_raymarch(ctx_.get(), &params, d.data(), t.data(), nullptr, static_cast<float*>(rgba.data()),
                                 static_cast<float*>(depth.data()), nullptr));
        Image img;
        img.width = params.width;
        img.height = params.height;
        img.rgba.resize(px * 4);
        img.depth.resize(px);
        rgba.download(img.rgba.data(), px * 16);
        depth.download(img.depth.data(), px * 4);
        ctx_.sync();
        return img;
    }

private:
    cuda::Context& ctx_;
};

// The per-pixel linked list of the colour pass (include/vkhr/rasterizer/
// linked_list.hh, src/vkhr/rasterizer/linked_list.cc) without Vulkan.  The
// colour image is width*height RGBA8 words (red in the low byte): the
// background going in, the resolved frame coming out.
class LinkedList {
public:
    static constexpr std::size_t AverageFragmentsPerPixel = 32; // linked_list.hh:28
    static constexpr std::size_t NodeSize = 12;                  // ppll.glsl's Node
    static constexpr std::uint32_t Null = VKHR_PPLL_NULL;

    LinkedList(cuda::Context& ctx, std::uint32_t width, std::uint32_t height)
        : ctx_(ctx), width_(width), height_(height)
    {
    }

    std::uint32_t width() const { return width_; }
    std::uint32_t height() const { return height_; }

    // resolve.comp over a PPLL: `heads` (width*height, Null = empty) and `nodes`.
    std::vector<std::uint32_t> resolve(const std::vector<std::uint32_t>& heads,
                                       const std::vector<vkhr_ppll_node>& nodes,
                                       const std::vector<std::uint32_t>& color)
    {
        check_image(heads.size());
        check_image(color.size());
        cuda::Context::Buffer h = ctx_.upload(heads);
        cuda::Context::Buffer c = ctx_.upload(color);
        cuda::Context::Buffer n;
        if (!nodes.empty()) n = ctx_.upload(nodes);
        ctx_.check(vkhr_resolve_ppll(ctx_.get(), static_cast<const std::uint32_t*>(h.data()),
                                     static_cast<const vkhr_ppll_node*>(n.data()), (std::uint32_t)nodes.size(),
                                     (std::int32_t)width_, (std::int32_t)height_,
                                     static_cast<std::uint32_t*>(c.data()), nullptr));
        return finish(c);
    }

    // The same step without lists: strand fragments in the order they were
    // emitted, and optionally the raymarched volume's fragments (a pixel holds
    // one where its depth is below 1), resolved as if linked in that order.
    std::vector<std::uint32_t> composite(const std::vector<vkhr_fragment>& fragments,
                                         const std::vector<std::uint32_t>& color,
                                         const Raymarcher::Image* volume = nullptr)
    {
        check_image(color.size());
        cuda::Context::Buffer c = ctx_.upload(color);
        cuda::Context::Buffer f, vr, vd;
        if (!fragments.empty()) f = ctx_.upload(fragments);
        if (volume) {
            if ((std::uint32_t)volume->width != width_ || (std::uint32_t)volume->height != height_)
                throw cuda::Error(VKHR_ERR_INVALID_ARG, "LinkedList::composite: volume image size differs");
            vr = ctx_.upload(volume->rgba);
            vd = ctx_.upload(volume->depth);
        }
        ctx_.check(vkhr_composite(ctx_.get(), static_cast<const vkhr_fragment*>(f.data()),
                                  (std::uint32_t)fragments.size(), static_cast<const float*>(vr.data()),
                                  static_cast<const float*>(vd.data()), (std::int32_t)width_, (std::int32_t)height_,
                                  static_cast<std::uint32_t*>(c.data()), nullptr));
        return finish(c);
    }

private:
    void check_image(std::size_t n) const
    {
        if (n != (std::size_t)width_ * height_)
            throw cuda::Error(VKHR_ERR_INVALID_ARG, "LinkedList: an image array is not width * height long");
    }

    std::vector<std::uint32_t> finish(const cuda::Context::Buffer& c)
    {
        std::vector<std::uint32_t> out((std::size_t)width_ * height_);
        c.download(out.data(), out.size() * sizeof(std::uint32_t));
        ctx_.check(vkhr_check_status(ctx_.get(), nullptr)); // waits; reports indices out of range
        return out;
    }

    cuda::Context& ctx_;
    std::uint32_t width_, height_;
};

} // namespace vkhr

#endif
