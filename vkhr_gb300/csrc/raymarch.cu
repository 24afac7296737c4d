// raymarch.cu -- volume raymarcher: the proxy-cube entry, isosurface march,
// Kajiya-Kay shading, density self-shadowing and local ambient occlusion of
// share/shaders/volumes/volume.frag:31-103 and its includes, in FP32 on GB300.
//
// One thread per pixel; a warp covers an 8x4 pixel tile so that neighbouring
// rays walk neighbouring voxels.  Differences from a literal translation, all
// exact with respect to the shader's outputs:
//   * the proxy cube's rasterization becomes a slab test of the pixel-centre
//     ray against the AABB (front faces only: a camera inside covers nothing);
//   * the per-step depth test (volume_rendering.glsl:30-34) is skipped when
//     the ray's far end already passes it (depth grows monotonically along a
//     ray that moves away from the camera);
//   * the primary march stops once the isosurface point is frozen
//     (acc > iso), found, and coverage lod*(acc/iso)*alpha >= 1, after which
//     no later sample can change any output (coverage is clamped to 1);
//   * texture filtering is a software trilinear with FP32 weights at Vulkan's
//     texel centres, CLAMP_TO_BORDER reading 0.
#include "march.cuh"

#include <cuda.h> // CUtensorMap and its enums (the encoder is looked up in the driver at run time)

#include <mutex>

namespace {

// Ray packets: a warp marches a TW x (32 / TW) pixel tile, and MINB
// resident CTAs per SM are asked for (6: at most 85 registers per thread,
// 8: at most 64).  The
// variants compute the same pixels; the autotuner picks one per context
// and texel format.
struct RayVariant {
    int tw, minb;
};
constexpr int kPacketVariants = 4;   // raymarch_kernel instantiations; variant 4 is the staged kernel
constexpr int kStagedVariant = 4;
constexpr int kTextureVariant = 5;   // the texture unit's filter: other pixels, never autotuned
constexpr int kShadeTextureVariant = 6; // the same filter for the shading's samples only
constexpr int kGatherVariant = 7;    // exact texels by texture gathers: the same pixels
constexpr int kGroup4Variant = 8;    // ray groups of 4 lanes, 4x2-pixel warp tiles: the same pixels
constexpr int kGroup2Variant = 9;    // ray groups of 2 lanes, 4x4-pixel warp tiles: the same pixels
constexpr int kGroup8Variant = 10;   // ray groups of 8 lanes, 2x2-pixel warp tiles: the same pixels
// the variants that compute the same pixels (the autotuner's candidates)
constexpr int kTunedVariants[] = {0, 1, 2, 3, 4, kGatherVariant, kGroup4Variant, kGroup2Variant, kGroup8Variant};
static_assert(VKHR_RAYMARCH_VARIANTS == kGroup8Variant + 1, "variant table");
constexpr RayVariant kRayVariants[kPacketVariants] = {{8, 6}, {16, 6}, {4, 6}, {8, 8}};

template <int DF, int TF, int TW = 8, int MINB = 6, int SRC = kSampleMemory>
__global__ void __launch_bounds__(32 * kWarpsX * kWarpsY, MINB)
raymarch_kernel(const __grid_constant__ RayConsts c, const typename DensityTexel<DF>::T* __restrict__ dens,
                const void* __restrict__ tang, const uint32_t* __restrict__ occ, const float* __restrict__ depth_in,
                float4* __restrict__ rgba, float* __restrict__ depth_out, int x0, int y0, int x1, int y1)
{
    // the pixels [x0, x1) x [y0, y1): the volume's footprint (background_kernel writes the rest)
    constexpr int TH = 32 / TW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = x0 + (blockIdx.x * kWarpsX + (warp % kWarpsX)) * TW + (lane % TW);
    const int py = y0 + (blockIdx.y * kWarpsY + (warp / kWarpsX)) * TH + (lane / TW);
    if (px >= x1 || py >= y1) return;
    const size_t at = (size_t)py * c.W + px;
    float4 out;
    float out_depth;
    march_pixel<DF, TF, false, SRC>(c, dens, tang, occ, depth_in ? depth_in + at : nullptr, px, py, out, out_depth);
    rgba[at] = out;
    if (depth_out) depth_out[at] = out_depth;
}

// Ray groups: G lanes march each pixel's ray (march_pixel's group form), a
// warp's 32 / G pixels as a TW x (32 / G / TW) tile; the group's first lane
// writes the pixel.
template <int DF, int TF, int G, int TW>
__global__ void __launch_bounds__(32 * kWarpsX * kWarpsY, 6)
raymarch_group_kernel(const __grid_constant__ RayConsts c, const typename DensityTexel<DF>::T* __restrict__ dens,
                      const void* __restrict__ tang, const uint32_t* __restrict__ occ,
                      const float* __restrict__ depth_in, float4* __restrict__ rgba, float* __restrict__ depth_out,
                      int x0, int y0, int x1, int y1)
{
    constexpr int TH = 32 / G / TW;
    static_assert(TW * TH * G == 32, "a warp's tile");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, pix = lane / G;
    const int px = x0 + (blockIdx.x * kWarpsX + (warp % kWarpsX)) * TW + (pix % TW);
    const int py = y0 + (blockIdx.y * kWarpsY + (warp / kWarpsX)) * TH + (pix / TW);
    if (px >= x1 || py >= y1) return; // the whole group: its lanes share the pixel
    const size_t at = (size_t)py * c.W + px;
    float4 out;
    float out_depth;
    march_pixel<DF, TF, false, kSampleMemory, G>(c, dens, tang, occ, depth_in ? depth_in + at : nullptr, px, py, out,
                                                 out_depth);
    if ((lane & (G - 1)) == 0) {
        rgba[at] = out;
        if (depth_out) depth_out[at] = out_depth;
    }
}

// ---- TMA-staged primary march ----------------------------------------------------
// raymarch_kernel with the primary march's density texels read from shared
// memory.  Each warp marches its 8x4 rays in rounds: every live ray advances
// through the samples that need no texel (exactly zero in an empty brick,
// jumped as in march_pixel) to its next sample in an occupied brick; the warp
// takes the brick the first such ray needs, one lane loads the brick's texels
// -- cells [8b, 8b + 8) reach texels [8b - 1, 8b + 7] per axis -- with one
// cp.async.bulk.tensor.3d into the warp's slot (the tensor map's zero fill
// outside the grid is the sampler's border 0), and every ray whose sample lies
// in that brick takes its samples from the slot until it leaves the brick.
// The samples, their order and their arithmetic are march_pixel's, so the
// image is the same bit for bit; shading (tangent, shadows, AO) reads global
// memory as before.  Needs a tensor map of the density grid (row pitch a
// multiple of 16 bytes, 16-byte aligned base).

template <int DF>
struct Stage {
    typedef typename DensityTexel<DF>::T T;
    static constexpr int kAlign = 16 / (int)sizeof(T); // a box's x start is a whole 16 bytes
    // x extent from the aligned start down from 8b - 1 through 8b + 7, in whole 16 bytes
    static constexpr int kX = sizeof(T) == 1 ? 32 : 12;
    static constexpr int kY = 9, kZ = 9;
    static constexpr uint32_t kBytes = (uint32_t)(kX * kY * kZ * sizeof(T));
    static constexpr uint32_t kSlot = (kBytes + 127u) / 128u * 128u;
};
constexpr int kStageWarps = kWarpsX * kWarpsY;
constexpr uint32_t kStageWaitLimit = 1u << 20; // try_wait rounds before a brick load counts as lost

template <int DF>
constexpr size_t staged_smem_bytes() { return (size_t)kStageWarps * (Stage<DF>::kSlot + 8); }

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n\tfence.mbarrier_init.release.cluster;" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < kStageWaitLimit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// One lane: the box of brick b's texels, origin (ox, oy, oz), into the slot.
__device__ __forceinline__ void load_box(const CUtensorMap* map, uint32_t slot, uint32_t bar, uint32_t bytes, int ox,
                                         int oy, int oz)
{
    // the warp's earlier reads of the slot (generic proxy) before the copy's writes (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                 ::"r"(slot), "l"(reinterpret_cast<uint64_t>(map)), "r"(ox), "r"(oy), "r"(oz), "r"(bar)
                 : "memory");
}

// sample_density from the staged box (origin ox, oy, oz) of the sample's brick.
template <int DF>
__device__ __forceinline__ float sample_box(const RayConsts& c, const typename DensityTexel<DF>::T* box, int ox, int oy,
                                            int oz, Vec3 p)
{
    typedef Stage<DF> S;
    int i0[3];
    float a[3];
    tex_setup(c, p, i0, a); // true for every sample inside the cell grid
    constexpr int sy = S::kX, sz = S::kX * S::kY;
    const int b = ((i0[2] - oz) * S::kY + (i0[1] - oy)) * S::kX + (i0[0] - ox);
    float v[8];
    v[0] = (float)box[b];
    v[1] = (float)box[b + 1];
    v[2] = (float)box[b + sy];
    v[3] = (float)box[b + sy + 1];
    v[4] = (float)box[b + sz];
    v[5] = (float)box[b + sz + 1];
    v[6] = (float)box[b + sz + sy];
    v[7] = (float)box[b + sz + sy + 1];
    const float x00 = fmaf(a[0], v[1] - v[0], v[0]);
    const float x10 = fmaf(a[0], v[3] - v[2], v[2]);
    const float x01 = fmaf(a[0], v[5] - v[4], v[4]);
    const float x11 = fmaf(a[0], v[7] - v[6], v[6]);
    const float y0 = fmaf(a[1], x10 - x00, x00);
    const float y1 = fmaf(a[1], x11 - x01, x01);
    return fmaf(a[2], y1 - y0, y0) * DensityTexel<DF>::scale;
}

__device__ __forceinline__ int floor_to(int x, int m) { return (x >= 0 ? x / m : -((-x + m - 1) / m)) * m; }

template <int DF, int TF>
__global__ void __launch_bounds__(32 * kWarpsX * kWarpsY, 6)
raymarch_staged_kernel(const __grid_constant__ RayConsts c, const __grid_constant__ CUtensorMap map,
                       const typename DensityTexel<DF>::T* __restrict__ dens, const void* __restrict__ tang,
                       const uint32_t* __restrict__ occ, const float* __restrict__ depth_in,
                       float4* __restrict__ rgba, float* __restrict__ depth_out, int x0, int y0, int x1, int y1,
                       unsigned long long* __restrict__ words)
{
    typedef Stage<DF> S;
    typedef typename DensityTexel<DF>::T T;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T* box = reinterpret_cast<const T*>(smem + (size_t)warp * S::kSlot);
    const uint32_t slot = smem_addr(box);
    const uint32_t bar = smem_addr(smem + (size_t)kStageWarps * S::kSlot + 8 * warp);
    if (lane == 0) mbar_init(bar);
    __syncwarp();

    // the warp's 8x4 pixels, as raymarch_kernel's default packet; every lane
    // stays to the end (the warp loads bricks together)
    const int px = x0 + (blockIdx.x * kWarpsX + (warp % kWarpsX)) * kTileW + (lane % kTileW);
    const int py = y0 + (blockIdx.y * kWarpsY + (warp / kWarpsX)) * kTileH + (lane / kTileW);
    const bool valid = px < x1 && py < y1;
    const size_t at = valid ? (size_t)py * c.W + px : 0;
    Vec3 start = v3(0.0f, 0.0f, 0.0f), end = start;
    const bool hit = valid && ray_entry(c, px, py, start, end);
    const float db = (hit && depth_in) ? depth_in[at] : 1.0f;
    const bool depth_test = hit && !(clip_depth(c, end) < db);
    const float step = 1.0f / c.steps;
    const bool jump = c.steps_pow2 && !depth_test;
    float inv_du[3] = {0.0f, 0.0f, 0.0f};
    if (hit) {
        float us[3], ue[3], du[3];
        texel_coords(c, start, us);
        texel_coords(c, end, ue);
        du[0] = ue[0] - us[0];
        du[1] = ue[1] - us[1];
        du[2] = ue[2] - us[2];
        reciprocals(du, inv_du);
    }
    float t = 0.0f, acc = 0.0f;
    Vec3 surf = v3(0.0f, 0.0f, 0.0f), entry = surf;
    bool found = false, entered = false, live = hit, lost = false;
    uint32_t parity = 0;
    for (;;) {
        // ---- to the ray's next sample that reads texels (volume_rendering.glsl:28-47)
        int need = -1;
        while (live) {
            if (!(t < 1.0f)) {
                live = false;
                break;
            }
            const Vec3 P = mix(start, end, t);
            if (depth_test && db < clip_depth(c, P)) {
                live = false;
                break;
            }
            float u[3], lo[3], hi[3];
            texel_coords(c, P, u);
            const int z = classify(c, occ, u, inv_du, lo, hi);
            if (z == 2) {
                live = false;
                break;
            }
            if (z == 1) {
                const float n = jump ? steps_inside(u, inv_du, lo, hi, c.steps) : 0.0f;
                t = n >= 1.0f ? fmaf(n, step, t) : t + step;
                continue;
            }
            need = (int)cell_brick(c, u);
            break;
        }
        const unsigned want = __ballot_sync(0xffffffffu, need >= 0);
        if (!want) break;
        // ---- the brick of the first waiting ray, staged
        const int b = __shfl_sync(0xffffffffu, need, __ffs(want) - 1);
        const int bx = b % c.nb[0], by = (b / c.nb[0]) % c.nb[1], bz = b / (c.nb[0] * c.nb[1]);
        const int ox = floor_to(kBrick * bx - 1, S::kAlign), oy = kBrick * by - 1, oz = kBrick * bz - 1;
        if (lane == 0) load_box(&map, slot, bar, S::kBytes, ox, oy, oz);
        const bool arrived = mbar_wait(bar, parity);
        if (__any_sync(0xffffffffu, !arrived)) { // a load that never lands: report it and stop marching
            if (lane == 0) {
                atomicOr(words + WORD_STATUS, (unsigned long long)VKHR_DEV_TIMEOUT);
                mbar_wait(bar, parity); // give the copy one more bounded wait before the slot is let go
            }
            lost = true;
            break;
        }
        parity ^= 1u;
        // ---- the samples of the rays inside that brick
        if (need == b) {
            for (;;) {
                const Vec3 P = mix(start, end, t);
                const float rho = sample_box<DF>(c, box, ox, oy, oz, P);
                acc += rho;
                if (rho != 0.0f) {
                    if (acc <= c.iso) surf = P;
                    if (acc >= c.iso) found = true;
                    if (!entered) {
                        entry = P;
                        entered = true;
                    }
                    if (acc > c.iso && c.lod * (acc / c.iso) * c.alpha >= 1.0f) { // outputs final
                        live = false;
                        break;
                    }
                }
                t += step;
                if (!(t < 1.0f)) {
                    live = false;
                    break;
                }
                const Vec3 Q = mix(start, end, t);
                if (depth_test && db < clip_depth(c, Q)) {
                    live = false;
                    break;
                }
                float u[3], lo[3], hi[3];
                texel_coords(c, Q, u);
                if (classify(c, occ, u, inv_du, lo, hi) != 0 || (int)cell_brick(c, u) != b) break;
            }
        }
        __syncwarp(); // every lane is done with the slot before the next load
    }
    if (!valid) return;
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float out_depth = 1.0f;
    if (hit && !lost) {
        if (!found && entered) surf = entry;
        shade_fragment<DF, TF>(c, dens, tang, occ, surf, acc, out, out_depth);
    }
    rgba[at] = out;
    if (depth_out) depth_out[at] = out_depth;
}

// Background (RGBA 0, depth 1: what march_pixel gives a ray that misses the
// volume's box) for the pixels outside [x0, x1) x [y0, y1).  A pixel outside
// the footprint rectangle misses the box, so the march launch covers the
// rectangle only instead of one CTA per tile of the whole view.
__global__ void background_kernel(float4* __restrict__ rgba, float* __restrict__ depth, int W, int H, int x0, int y0,
                                  int x1, int y1)
{
    const size_t n = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int py = (int)(i / (size_t)W), px = (int)(i - (size_t)py * W);
        if (px >= x0 && px < x1 && py >= y0 && py < y1) continue;
        rgba[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (depth) depth[i] = 1.0f;
    }
}

// ---- batched raymarch ------------------------------------------------------------
// Many views (one style each) in one persistent launch.  Each job renders a
// rectangular region of its own view; the regions' tiles form one index
// space that CTAs pull from a device queue, most expensive jobs first.

constexpr int kMaxRayJobs = 256;
constexpr int kRegionTileW = kTileW * kWarpsX, kRegionTileH = kTileH * kWarpsY;

struct RayJob {
    RayConsts c;
    const void* dens;
    const void* tang;
    const float* depth_in; // region layout, may be NULL
    float4* rgba;          // region layout: pixel (x0 + i, y0 + j) at [j * pitch + i]
    float* depth_out;      // may be NULL
    uint32_t* occ;         // this view's occupancy bitmap
    int x0, y0, w, h, pitch, tiles_x;
    uint32_t tile_base;    // first tile of the job in the batch
    uint32_t column_base;  // first occupancy column of the job's volume in the batch
};

static_assert(sizeof(RayJob) % 4 == 0, "RayJob is copied as 32-bit words");
static_assert(sizeof(RayJob) * kMaxRayJobs <= kRayTableBytes, "raymarch job table staging too small");

// Largest j with base[j] <= x (base ascending, base[0] = 0).
__device__ __forceinline__ int find_base(const uint32_t* base, int nj, uint32_t x)
{
    int lo = 0, hi = nj - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int DF>
__global__ void occupancy_batched_kernel(const RayJob* __restrict__ jobs, int nj, uint32_t total_columns)
{
    __shared__ uint32_t s_base[kMaxRayJobs];
    for (int j = threadIdx.x; j < nj; j += blockDim.x) s_base[j] = jobs[j].column_base;
    __syncthreads();
    // one thread per column (a batch has columns enough to fill the GPU)
    const uint64_t lanes = total_columns, stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < lanes; g += stride) {
        const bool valid = true;
        const uint32_t i = (uint32_t)g;
        const RayJob& J = jobs[find_base(s_base, nj, i)];
        const uint32_t li = i - J.column_base;
        const int nx = J.c.res[0], ny = J.c.res[1], nz = J.c.res[2];
        const uint32_t cxn = (uint32_t)(nx + 7) / 8, an = (uint32_t)(ny + 7) / 8;
        const uint32_t r = li / cxn, cx = li - r * cxn, c = r / an, a = r - c * an;
        occupancy_column<DF, 1>((const typename DensityTexel<DF>::T*)J.dens, nx, ny, nz, J.c.nb[0], J.c.nb[1], J.occ,
                                (int)cx, (int)a, (int)c, valid);
    }
}

template <int DF, int TF>
__global__ void __launch_bounds__(32 * kWarpsX * kWarpsY)
raymarch_batched_kernel(const RayJob* __restrict__ jobs, int nj, uint32_t total_tiles, unsigned long long* words)
{
    __shared__ RayJob sj;
    __shared__ uint32_t s_base[kMaxRayJobs];
    __shared__ uint32_t s_next;
    for (int j = threadIdx.x; j < nj; j += blockDim.x) s_base[j] = jobs[j].tile_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lx = (warp % kWarpsX) * kTileW + (lane % kTileW), ly = (warp / kWarpsX) * kTileH + (lane / kTileW);
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) s_next = (uint32_t)atomicAdd(words + WORD_RAY_QUEUE, 1ull);
        __syncthreads();
        const uint32_t tile = s_next;
        __syncthreads();
        if (tile >= total_tiles) break;
        const int j = find_base(s_base, nj, tile);
        if (j != cur) { // every thread finished the previous tile before the barrier above
            const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + j);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&sj);
            for (int i = threadIdx.x; i < (int)(sizeof(RayJob) / 4); i += blockDim.x) dst[i] = __ldg(src + i);
            __syncthreads();
            cur = j;
        }
        const uint32_t t = tile - sj.tile_base;
        const int rx = (int)(t % (uint32_t)sj.tiles_x) * kRegionTileW + lx;
        const int ry = (int)(t / (uint32_t)sj.tiles_x) * kRegionTileH + ly;
        if (rx < sj.w && ry < sj.h) {
            const size_t at = (size_t)ry * sj.pitch + rx;
            float4 out;
            float out_depth;
            march_pixel<DF, TF>(sj.c, (const typename DensityTexel<DF>::T*)sj.dens, sj.tang, sj.occ,
                                sj.depth_in ? sj.depth_in + at : nullptr, sj.x0 + rx, sj.y0 + ry, out, out_depth);
            sj.rgba[at] = out;
            if (sj.depth_out) sj.depth_out[at] = out_depth;
        }
    }
}

// The density as a 3D texture for the texture-unit variant: a CUDA array of
// the grid's extent (kept in the context, re-made when the extent or format
// changes), LINEAR filtering, border 0 (CLAMP_TO_BORDER), u8 read as UNORM;
// the call copies the density into it on the stream.  Integer counts cannot
// be filtered by the texture unit (false: the caller marches from memory).
template <int DF>
vkhr_status texture_density(vkhr_ctx* ctx, const RayConsts& c, const void* dens, cudaStream_t st, bool& ok)
{
    ok = false;
    if (DF == VKHR_DENSITY_U32_COUNT) return VKHR_OK;
    const size_t es = sizeof(typename DensityTexel<DF>::T);
    if (!ctx->tex_array || ctx->tex_fmt != DF || ctx->tex_res[0] != c.res[0] || ctx->tex_res[1] != c.res[1] ||
        ctx->tex_res[2] != c.res[2]) {
        if (ctx->tex_array && ctx->live_graphs > 0)
            return vkhr_fail(ctx, VKHR_ERR_CAPACITY, "the density texture would have to change while a frame graph lives");
        if (ctx->tex_obj) cudaDestroyTextureObject(ctx->tex_obj);
        if (ctx->tex_array) {
            VKHR_CUDA_TRY(ctx, cudaDeviceSynchronize()); // earlier launches may still read it
            cudaFreeArray(ctx->tex_array);
        }
        ctx->tex_obj = 0;
        ctx->tex_array = nullptr;
        const cudaChannelFormatDesc fd =
            DF == VKHR_DENSITY_U8_UNORM ? cudaCreateChannelDesc<unsigned char>() : cudaCreateChannelDesc<float>();
        VKHR_CUDA_TRY(ctx, cudaMalloc3DArray(&ctx->tex_array, &fd, make_cudaExtent(c.res[0], c.res[1], c.res[2])));
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = ctx->tex_array;
        cudaTextureDesc td = {};
        for (int k = 0; k < 3; ++k) td.addressMode[k] = cudaAddressModeBorder; // border colour 0
        td.filterMode = cudaFilterModeLinear;
        td.readMode = DF == VKHR_DENSITY_U8_UNORM ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
        td.normalizedCoords = 0;
        VKHR_CUDA_TRY(ctx, cudaCreateTextureObject(&ctx->tex_obj, &rd, &td, nullptr));
        for (int k = 0; k < 3; ++k) ctx->tex_res[k] = c.res[k];
        ctx->tex_fmt = DF;
    }
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr(const_cast<void*>(dens), (size_t)c.res[0] * es, (size_t)c.res[0], (size_t)c.res[1]);
    cp.dstArray = ctx->tex_array;
    cp.extent = make_cudaExtent(c.res[0], c.res[1], c.res[2]);
    cp.kind = cudaMemcpyDeviceToDevice;
    VKHR_CUDA_TRY(ctx, cudaMemcpy3DAsync(&cp, st));
    ok = true;
    return VKHR_OK;
}

// The gather variant's texture: the grid's z slices tiled 2^shift per row
// into a 2D array, each slice framed by zeros (see sample_density_gather).
// One thread per texel of the array, a block row per array row (blockIdx.y);
// written through a surface of the array when it has one, else into a
// linear staging buffer (row pitch `width` texels) that is copied in after.
template <typename T>
__global__ void gather_tile_kernel(const T* __restrict__ src, cudaSurfaceObject_t surf, T* __restrict__ dst, int nx,
                                   int ny, int nz, int shift, uint32_t width)
{
    const uint32_t X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
    if (X >= width) return;
    const uint32_t tw = (uint32_t)nx + 2, th = (uint32_t)ny + 2;
    const uint32_t tx = X / tw, ty = Y / th;
    const int x = (int)(X - tx * tw) - 1, y = (int)(Y - ty * th) - 1;
    const int z = (int)((ty << shift) + tx);
    T v = T(0);
    if (x >= 0 && x < nx && y >= 0 && y < ny && z < nz)
        v = __ldg(src + (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z));
    if (surf) surf2Dwrite(v, surf, (int)(X * sizeof(T)), (int)Y);
    else dst[(size_t)Y * width + X] = v;
}

// Copies the density into the context's gather texture (allocated, or
// reallocated when the grid or format changes); false (ok) when the tiled
// slices exceed the texture unit's gather limits.
template <int DF>
vkhr_status gather_density(vkhr_ctx* ctx, const RayConsts& c, const void* dens, cudaStream_t st, bool& ok)
{
    typedef typename DensityTexel<DF>::T T;
    ok = false;
    int shift = 0;
    while ((1 << shift) * (1 << shift) < c.res[2]) ++shift; // 2^shift >= sqrt(depth)
    const uint64_t per_row = 1ull << shift, rows = ((uint64_t)c.res[2] + per_row - 1) / per_row;
    const uint64_t width = per_row * ((uint64_t)c.res[0] + 2), height = rows * ((uint64_t)c.res[1] + 2);
    int max_w = 0, max_h = 0;
    VKHR_CUDA_TRY(ctx, cudaDeviceGetAttribute(&max_w, cudaDevAttrMaxTexture2DGatherWidth, ctx->device));
    VKHR_CUDA_TRY(ctx, cudaDeviceGetAttribute(&max_h, cudaDevAttrMaxTexture2DGatherHeight, ctx->device));
    if (width > (uint64_t)max_w || height > (uint64_t)max_h) return VKHR_OK;
    if (!ctx->gat_array || ctx->gat_fmt != DF || ctx->gat_res[0] != c.res[0] || ctx->gat_res[1] != c.res[1] ||
        ctx->gat_res[2] != c.res[2]) {
        if (ctx->gat_array && ctx->live_graphs > 0)
            return vkhr_fail(ctx, VKHR_ERR_CAPACITY, "the density texture would have to change while a frame graph lives");
        if (ctx->gat_obj) cudaDestroyTextureObject(ctx->gat_obj);
        if (ctx->gat_array) {
            VKHR_CUDA_TRY(ctx, cudaDeviceSynchronize()); // earlier launches may still read it
            cudaFreeArray(ctx->gat_array);
        }
        if (ctx->gat_surf) cudaDestroySurfaceObject(ctx->gat_surf);
        ctx->gat_obj = 0;
        ctx->gat_surf = 0;
        ctx->gat_array = nullptr;
        const cudaChannelFormatDesc fd = cudaCreateChannelDesc<T>();
        // writable as a surface where the driver allows it with gathers, else filled by a copy
        bool surface = true;
        if (cudaMallocArray(&ctx->gat_array, &fd, (size_t)width, (size_t)height,
                            cudaArrayTextureGather | cudaArraySurfaceLoadStore) != cudaSuccess) {
            cudaGetLastError();
            surface = false;
            VKHR_CUDA_TRY(ctx, cudaMallocArray(&ctx->gat_array, &fd, (size_t)width, (size_t)height,
                                               cudaArrayTextureGather));
        }
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = ctx->gat_array;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder; // border colour 0
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        VKHR_CUDA_TRY(ctx, cudaCreateTextureObject(&ctx->gat_obj, &rd, &td, nullptr));
        if (surface) VKHR_CUDA_TRY(ctx, cudaCreateSurfaceObject(&ctx->gat_surf, &rd));
        for (int k = 0; k < 3; ++k) ctx->gat_res[k] = c.res[k];
        ctx->gat_fmt = DF;
        ctx->gat_shift = shift;
    }
    if (!ctx->gat_surf) {
        vkhr_status s = vkhr_reserve(ctx, &ctx->gat_stage, &ctx->gat_stage_cap, (size_t)(width * height * sizeof(T)), 1);
        if (s != VKHR_OK) return s;
    }
    const dim3 grid((unsigned)((width + 255) / 256), (unsigned)height);
    VKHR_LAUNCH(ctx, gather_tile_kernel<T>, grid, 256, 0, st, (const T*)dens, ctx->gat_surf, (T*)ctx->gat_stage,
                c.res[0], c.res[1], c.res[2], shift, (uint32_t)width);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    if (!ctx->gat_surf)
        VKHR_CUDA_TRY(ctx, cudaMemcpy2DToArrayAsync(ctx->gat_array, 0, 0, ctx->gat_stage, (size_t)width * sizeof(T),
                                                    (size_t)width * sizeof(T), (size_t)height, cudaMemcpyDeviceToDevice,
                                                    st));
    ok = true;
    return VKHR_OK;
}

// cuTensorMapEncodeTiled from the driver (looked up once; NULL if unavailable).
typedef CUresult (*TensorMapEncoder)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                     const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

TensorMapEncoder tensor_map_encoder()
{
    static std::once_flag once;
    static TensorMapEncoder fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<TensorMapEncoder>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// The tensor map of a density grid for the staged march: 3D, the grid's own
// extent (texels outside it read as zero), box Stage<DF>::kX x 9 x 9.  False
// when TMA cannot address the grid: a base not 16-byte aligned, or a row
// pitch not a multiple of 16 bytes.
template <int DF>
bool density_tensor_map(const RayConsts& c, const void* dens, CUtensorMap* map)
{
    typedef Stage<DF> S;
    const size_t es = sizeof(typename S::T);
    const TensorMapEncoder enc = tensor_map_encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(dens) & 15u) || ((size_t)c.res[0] * es) % 16 != 0) return false;
    const CUtensorMapDataType type = DF == VKHR_DENSITY_U8_UNORM ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                     : DF == VKHR_DENSITY_U32_COUNT ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                                                                    : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const cuuint64_t dim[3] = {(cuuint64_t)c.res[0], (cuuint64_t)c.res[1], (cuuint64_t)c.res[2]};
    const cuuint64_t stride[2] = {(cuuint64_t)c.res[0] * es, (cuuint64_t)c.res[0] * c.res[1] * es};
    const cuuint32_t box[3] = {(cuuint32_t)S::kX, (cuuint32_t)S::kY, (cuuint32_t)S::kZ};
    const cuuint32_t elem[3] = {1, 1, 1};
    return enc(map, type, 3, const_cast<void*>(dens), dim, stride, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int DF, int TF>
vkhr_status launch(vkhr_ctx* ctx, const RayConsts& c, const void* dens, const void* tang, const float* din, float* rgba,
                   float* dout, const int32_t rect[4], cudaStream_t st)
{
    const size_t bricks = (size_t)c.nb[0] * c.nb[1] * c.nb[2];
    const size_t words = (bricks + 31) / 32;
    vkhr_status s = vkhr_reserve(ctx, (void**)&ctx->occ, &ctx->occ_cap, words, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->occ, 0, words * sizeof(uint32_t), st));
    {
        const typename DensityTexel<DF>::T* dd = (const typename DensityTexel<DF>::T*)dens;
        const int L = occupancy_lanes(c.res[0], c.res[1], c.res[2], ctx->sm_count);
        const unsigned ob = occupancy_blocks(c.res[0], c.res[1], c.res[2], ctx->sm_count, L);
        if (L == 8)
            VKHR_LAUNCH(ctx, (occupancy_kernel<DF, 8>), ob, 128, 0, st, dd, c.res[0], c.res[1], c.res[2], c.nb[0], c.nb[1],
                        c.nb[2], ctx->occ);
        else
            VKHR_LAUNCH(ctx, (occupancy_kernel<DF, 1>), ob, 128, 0, st, dd, c.res[0], c.res[1], c.res[2], c.nb[0], c.nb[1],
                        c.nb[2], ctx->occ);
    }
    const int x0 = rect[0], y0 = rect[1], x1 = rect[0] + rect[2], y1 = rect[1] + rect[3];
    float4* out = reinterpret_cast<float4*>(rgba);
    const bool background = rect[2] < c.W || rect[3] < c.H;
    if (background) { // disjoint pixels: on the side stream, alongside the march
        s = vkhr_fork_side(ctx, st);
        if (s != VKHR_OK) return s;
        VKHR_LAUNCH(ctx, background_kernel, (unsigned)ctx->sm_count * 8, 256, 0, ctx->side, out, dout, c.W, c.H, x0, y0,
                    x1, y1);
    }
    if (rect[2] <= 0 || rect[3] <= 0) return background ? vkhr_join_side(ctx, st) : VKHR_OK;
    int v = ctx->ray_variant[DF][TF];
    const dim3 block(32 * kWarpsX * kWarpsY);
    if (v == kStagedVariant) {
        CUtensorMap map;
        if (density_tensor_map<DF>(c, dens, &map)) {
            const dim3 grid((rect[2] + kTileW * kWarpsX - 1) / (kTileW * kWarpsX),
                            (rect[3] + kTileH * kWarpsY - 1) / (kTileH * kWarpsY));
            VKHR_LAUNCH(ctx, (raymarch_staged_kernel<DF, TF>), grid, block, staged_smem_bytes<DF>(), st, c, map,
                        (const typename DensityTexel<DF>::T*)dens, tang, ctx->occ, din, out, dout, x0, y0, x1, y1,
                        ctx->d_words);
            return background ? vkhr_join_side(ctx, st) : VKHR_OK;
        }
        v = 0; // TMA cannot address this grid: the default packets
    }
    if (v == kTextureVariant || v == kShadeTextureVariant) {
        bool ok = false;
        vkhr_status ts = texture_density<DF>(ctx, c, dens, st, ok);
        if (ts != VKHR_OK) return ts;
        if (ok) {
            RayConsts ct = c;
            ct.tex = (unsigned long long)ctx->tex_obj;
            const dim3 grid((rect[2] + kTileW * kWarpsX - 1) / (kTileW * kWarpsX),
                            (rect[3] + kTileH * kWarpsY - 1) / (kTileH * kWarpsY));
            const typename DensityTexel<DF>::T* d = (const typename DensityTexel<DF>::T*)dens;
            if (v == kTextureVariant)
                VKHR_LAUNCH(ctx, (raymarch_kernel<DF, TF, 8, 6, kSampleTexture>), grid, block, 0, st, ct, d, tang,
                            ctx->occ, din, out, dout, x0, y0, x1, y1);
            else
                VKHR_LAUNCH(ctx, (raymarch_kernel<DF, TF, 8, 6, kSampleShadeTexture>), grid, block, 0, st, ct, d, tang,
                            ctx->occ, din, out, dout, x0, y0, x1, y1);
            return background ? vkhr_join_side(ctx, st) : VKHR_OK;
        }
        v = 0; // integer counts: the default packets
    }
    if (v == kGatherVariant) {
        bool ok = false;
        vkhr_status gs = gather_density<DF>(ctx, c, dens, st, ok);
        if (gs != VKHR_OK) return gs;
        if (ok) {
            RayConsts ct = c;
            ct.tex = (unsigned long long)ctx->gat_obj;
            ct.gshift = ctx->gat_shift;
            const dim3 grid((rect[2] + kTileW * kWarpsX - 1) / (kTileW * kWarpsX),
                            (rect[3] + kTileH * kWarpsY - 1) / (kTileH * kWarpsY));
            VKHR_LAUNCH(ctx, (raymarch_kernel<DF, TF, 8, 6, kSampleGather>), grid, block, 0, st, ct,
                        (const typename DensityTexel<DF>::T*)dens, tang, ctx->occ, din, out, dout, x0, y0, x1, y1);
            return background ? vkhr_join_side(ctx, st) : VKHR_OK;
        }
        v = 0; // beyond the gather limits: the default packets
    }
    const typename DensityTexel<DF>::T* d = (const typename DensityTexel<DF>::T*)dens;
    if (v == kGroup4Variant || v == kGroup2Variant || v == kGroup8Variant) { // 4x2 / 4x4 / 2x2 pixels per warp
        const int gw = v == kGroup8Variant ? 2 : 4, gh = v == kGroup2Variant ? 4 : 2;
        const dim3 grid((rect[2] + gw * kWarpsX - 1) / (gw * kWarpsX), (rect[3] + gh * kWarpsY - 1) / (gh * kWarpsY));
        if (v == kGroup4Variant)
            VKHR_LAUNCH(ctx, (raymarch_group_kernel<DF, TF, 4, 4>), grid, block, 0, st, c, d, tang, ctx->occ, din, out,
                        dout, x0, y0, x1, y1);
        else if (v == kGroup2Variant)
            VKHR_LAUNCH(ctx, (raymarch_group_kernel<DF, TF, 2, 4>), grid, block, 0, st, c, d, tang, ctx->occ, din, out,
                        dout, x0, y0, x1, y1);
        else
            VKHR_LAUNCH(ctx, (raymarch_group_kernel<DF, TF, 8, 2>), grid, block, 0, st, c, d, tang, ctx->occ, din, out,
                        dout, x0, y0, x1, y1);
        return background ? vkhr_join_side(ctx, st) : VKHR_OK;
    }
    const int tw = kRayVariants[v].tw, th = 32 / tw;
    const dim3 grid((rect[2] + tw * kWarpsX - 1) / (tw * kWarpsX), (rect[3] + th * kWarpsY - 1) / (th * kWarpsY));
#define VKHR_RAY(TW_, MINB_)                                                                                      \
    VKHR_LAUNCH(ctx, (raymarch_kernel<DF, TF, TW_, MINB_>), grid, block, 0, st, c, d, tang, ctx->occ, din, out, dout, x0, \
                y0, x1, y1)
    switch (v) {
    case 1: VKHR_RAY(16, 6); break;
    case 2: VKHR_RAY(4, 6); break;
    case 3: VKHR_RAY(8, 8); break;
    default: VKHR_RAY(8, 6);
    }
#undef VKHR_RAY
    return background ? vkhr_join_side(ctx, st) : VKHR_OK;
}

} // namespace

extern "C" vkhr_status vkhr_raymarch(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const void* d_density,
                                     const void* d_tangent, const float* d_depth_in, float* d_rgba, float* d_depth_out,
                                     void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!params || !d_density || !d_tangent || !d_rgba)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "params, d_density, d_tangent and d_rgba are required");
    if (reinterpret_cast<uintptr_t>(d_rgba) & 15u) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_rgba must be 16-byte aligned");
    RayConsts c;
    vkhr_status s = make_consts(ctx, params, c);
    if (s != VKHR_OK) return s;
    const size_t tan_align = params->tangent_format == VKHR_TANGENT_I8_SNORM ? 4 : 16;
    if (reinterpret_cast<uintptr_t>(d_tangent) & (tan_align - 1))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangent is misaligned for its format");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    int32_t rect[4]; // pixels outside it miss the volume's box
    s = vkhr_raymarch_footprint(params, rect);
    if (s != VKHR_OK) return vkhr_fail(ctx, s, "footprint of the view");
    const int df = params->density_format, tf = params->tangent_format;
    if (df == VKHR_DENSITY_U8_UNORM && tf == VKHR_TANGENT_I8_SNORM)
        s = launch<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_I8_SNORM>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    else if (df == VKHR_DENSITY_U8_UNORM)
        s = launch<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_F32X4>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    else if (df == VKHR_DENSITY_U32_COUNT && tf == VKHR_TANGENT_I8_SNORM)
        s = launch<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_I8_SNORM>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    else if (df == VKHR_DENSITY_U32_COUNT)
        s = launch<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_F32X4>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    else if (tf == VKHR_TANGENT_I8_SNORM)
        s = launch<VKHR_DENSITY_F32, VKHR_TANGENT_I8_SNORM>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    else
        s = launch<VKHR_DENSITY_F32, VKHR_TANGENT_F32X4>(ctx, c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, rect, st);
    if (s != VKHR_OK) return s; // e.g. scratch that could not grow: nothing was launched
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

extern "C" vkhr_status vkhr_set_raymarch_variant(vkhr_ctx* ctx, int32_t density_format, int32_t tangent_format,
                                                 int32_t variant)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (density_format < 0 || density_format > 2 || tangent_format < 0 || tangent_format > 1)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown texel format");
    if (variant < 0 || variant >= VKHR_RAYMARCH_VARIANTS) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown variant");
    ctx->ray_variant[density_format][tangent_format] = variant;
    return VKHR_OK;
}

extern "C" vkhr_status vkhr_autotune_raymarch(vkhr_ctx* ctx, const vkhr_raymarch_params* params, const void* d_density,
                                              const void* d_tangent, float* d_rgba, int32_t* chosen, float* variant_ms,
                                              void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!params || !chosen) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "params and chosen are required");
    const int df = params->density_format, tf = params->tangent_format;
    if (df < 0 || df > 2 || tf < 0 || tf > 1) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown texel format");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e[2];
    VKHR_CUDA_TRY(ctx, cudaEventCreate(&e[0]));
    if (cudaEventCreate(&e[1]) != cudaSuccess) {
        cudaEventDestroy(e[0]);
        return vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventCreate failed");
    }
    const int previous = ctx->ray_variant[df][tf];
    float ms[VKHR_RAYMARCH_VARIANTS];
    int best = 0;
    vkhr_status s = VKHR_OK;
    for (int v = 0; v < VKHR_RAYMARCH_VARIANTS; ++v) ms[v] = 0.0f;
    for (const int v : kTunedVariants) {
        if (s != VKHR_OK) break;
        ctx->ray_variant[df][tf] = v;
        float t[3] = {0.0f, 0.0f, 0.0f};
        for (int r = -1; r < 3 && s == VKHR_OK; ++r) { // one warm-up, three timed runs
            if (cudaEventRecord(e[0], st) != cudaSuccess) s = vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventRecord failed");
            if (s == VKHR_OK) s = vkhr_raymarch(ctx, params, d_density, d_tangent, nullptr, d_rgba, nullptr, stream);
            if (s == VKHR_OK && (cudaEventRecord(e[1], st) != cudaSuccess || cudaEventSynchronize(e[1]) != cudaSuccess))
                s = vkhr_fail(ctx, VKHR_ERR_CUDA, "timing the autotune runs failed");
            if (s == VKHR_OK && r >= 0 && cudaEventElapsedTime(&t[r], e[0], e[1]) != cudaSuccess)
                s = vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventElapsedTime failed");
        }
        std::sort(t, t + 3);
        ms[v] = t[1];
        if (ms[v] < ms[best]) best = v;
    }
    cudaEventDestroy(e[0]);
    cudaEventDestroy(e[1]);
    if (s != VKHR_OK) {
        ctx->ray_variant[df][tf] = previous;
        return s;
    }
    ctx->ray_variant[df][tf] = best;
    *chosen = best;
    if (variant_ms)
        for (int v = 0; v < VKHR_RAYMARCH_VARIANTS; ++v) variant_ms[v] = ms[v];
    return VKHR_OK;
}

// ---- batched raymarch: host side ------------------------------------------------------
namespace {

template <int DF, int TF>
vkhr_status launch_batched(vkhr_ctx* ctx, const RayJob* d_jobs, int nj, uint32_t total_columns, uint32_t total_tiles,
                           cudaStream_t st)
{
    const unsigned oblocks = (unsigned)std::min<size_t>((total_columns + 127) / 128, (size_t)ctx->sm_count * 16);
    if (total_columns)
        VKHR_LAUNCH(ctx, occupancy_batched_kernel<DF>, oblocks ? oblocks : 1, 128, 0, st, d_jobs, nj, total_columns);
    if (!total_tiles) return VKHR_OK;
    static int per_sm = 0; // resident CTAs per SM of this instantiation
    if (!per_sm) {
        int n = 0;
        VKHR_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, raymarch_batched_kernel<DF, TF>,
                                                                         32 * kWarpsX * kWarpsY, 0));
        per_sm = n > 0 ? n : 1;
    }
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)ctx->sm_count * per_sm, total_tiles);
    VKHR_LAUNCH(ctx, (raymarch_batched_kernel<DF, TF>), blocks, 32 * kWarpsX * kWarpsY, 0, st, d_jobs, nj,
                total_tiles, ctx->d_words);
    return VKHR_OK;
}

} // namespace

extern "C" vkhr_status vkhr_raymarch_batched(vkhr_ctx* ctx, const vkhr_raymarch_job* jobs, int32_t job_count,
                                             void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!jobs || job_count <= 0 || job_count > kMaxRayJobs)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "job count must be in [1, 256]");
    const int df = jobs[0].params.density_format, tf = jobs[0].params.tangent_format;
    // most expensive first: the queue hands out big jobs' tiles before small ones
    int order[kMaxRayJobs];
    double cost[kMaxRayJobs];
    for (int j = 0; j < job_count; ++j) {
        const vkhr_raymarch_job& in = jobs[j];
        if (!in.d_density || !in.d_tangent || !in.d_rgba)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_density, d_tangent and d_rgba are required");
        if (in.params.density_format != df || in.params.tangent_format != tf)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "every job of a batch uses the same texel formats");
        if (reinterpret_cast<uintptr_t>(in.d_rgba) & 15u)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_rgba must be 16-byte aligned");
        const size_t tan_align = tf == VKHR_TANGENT_I8_SNORM ? 4 : 16;
        if (reinterpret_cast<uintptr_t>(in.d_tangent) & (tan_align - 1))
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangent is misaligned for its format");
        if (in.w < 0 || in.h < 0 || in.x0 < 0 || in.y0 < 0 || (int64_t)in.x0 + in.w > in.params.width ||
            (int64_t)in.y0 + in.h > in.params.height || in.pitch < in.w)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "region outside the view, or pitch < region width");
        order[j] = j;
        cost[j] = (double)in.w * in.h * std::max(in.params.raycast_steps, 1.0f);
    }
    std::stable_sort(order, order + job_count, [&](int a, int b) { return cost[a] > cost[b]; });
    RayJob* table = reinterpret_cast<RayJob*>(ctx->h_rjobs);
    // the staging is reused once the previous batch's copy has run (not under capture: see below)
    cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (!capturing) VKHR_CUDA_TRY(ctx, cudaEventSynchronize(ctx->rjobs_ev));
    uint64_t tiles = 0, chunks = 0, words = 0;
    size_t occ_at[kMaxRayJobs];
    for (int k = 0; k < job_count; ++k) {
        const vkhr_raymarch_job& in = jobs[order[k]];
        RayJob& J = table[k];
        vkhr_status s = make_consts(ctx, &in.params, J.c);
        if (s != VKHR_OK) return s;
        J.dens = in.d_density;
        J.tang = in.d_tangent;
        J.depth_in = in.d_depth_in;
        J.rgba = reinterpret_cast<float4*>(in.d_rgba);
        J.depth_out = in.d_depth_out;
        J.x0 = in.x0;
        J.y0 = in.y0;
        J.w = in.w;
        J.h = in.h;
        J.pitch = in.pitch;
        J.tiles_x = (in.w + kRegionTileW - 1) / kRegionTileW;
        J.tile_base = (uint32_t)tiles;
        J.column_base = (uint32_t)chunks;
        tiles += (uint64_t)J.tiles_x * ((in.h + kRegionTileH - 1) / kRegionTileH);
        const uint64_t nb = (uint64_t)J.c.nb[0] * J.c.nb[1] * J.c.nb[2];
        chunks += occupancy_columns(J.c.res[0], J.c.res[1], J.c.res[2]);
        occ_at[k] = (size_t)words;
        words += (nb + 31) / 32;
        if (tiles >= (1ull << 32) || chunks >= (1ull << 32))
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "batch too large (2^32 tiles or texel chunks)");
    }
    vkhr_status s = vkhr_reserve(ctx, (void**)&ctx->occ, &ctx->occ_cap, (size_t)words, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    s = vkhr_reserve(ctx, &ctx->d_rjobs, &ctx->rjobs_cap, (size_t)job_count * sizeof(RayJob), 1);
    if (s != VKHR_OK) return s;
    for (int k = 0; k < job_count; ++k) table[k].occ = ctx->occ + occ_at[k];
    // Under capture the graph's copy reads the staging at every replay: the
    // staging then holds this table until the context's next raymarch batch.
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_rjobs, table, (size_t)job_count * sizeof(RayJob), cudaMemcpyHostToDevice,
                                       st));
    if (!capturing) VKHR_CUDA_TRY(ctx, cudaEventRecord(ctx->rjobs_ev, st));
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->occ, 0, (size_t)words * sizeof(uint32_t), st));
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words + WORD_RAY_QUEUE, 0, sizeof(unsigned long long), st));
    const RayJob* d_jobs = reinterpret_cast<const RayJob*>(ctx->d_rjobs);
    const uint32_t nbk = (uint32_t)chunks, nt = (uint32_t)tiles;
    if (df == VKHR_DENSITY_U8_UNORM && tf == VKHR_TANGENT_I8_SNORM)
        s = launch_batched<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_I8_SNORM>(ctx, d_jobs, job_count, nbk, nt, st);
    else if (df == VKHR_DENSITY_U8_UNORM)
        s = launch_batched<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_F32X4>(ctx, d_jobs, job_count, nbk, nt, st);
    else if (df == VKHR_DENSITY_U32_COUNT && tf == VKHR_TANGENT_I8_SNORM)
        s = launch_batched<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_I8_SNORM>(ctx, d_jobs, job_count, nbk, nt, st);
    else if (df == VKHR_DENSITY_U32_COUNT)
        s = launch_batched<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_F32X4>(ctx, d_jobs, job_count, nbk, nt, st);
    else if (tf == VKHR_TANGENT_I8_SNORM)
        s = launch_batched<VKHR_DENSITY_F32, VKHR_TANGENT_I8_SNORM>(ctx, d_jobs, job_count, nbk, nt, st);
    else
        s = launch_batched<VKHR_DENSITY_F32, VKHR_TANGENT_F32X4>(ctx, d_jobs, job_count, nbk, nt, st);
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

extern "C" vkhr_status vkhr_raymarch_footprint(const vkhr_raymarch_params* p, int32_t rect[4])
{
    if (!p || !rect || p->width <= 0 || p->height <= 0) return VKHR_ERR_INVALID_ARG;
    double pv[16];
    for (int col = 0; col < 4; ++col)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += (double)p->projection[k * 4 + r] * (double)p->view[col * 4 + k];
            pv[col * 4 + r] = s;
        }
    const double W = p->width, H = p->height;
    double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
    for (int k = 0; k < 8; ++k) {
        double x[4] = {p->volume_bounds.origin[0] + ((k & 1) ? p->volume_bounds.size[0] : 0.0f),
                       p->volume_bounds.origin[1] + ((k & 2) ? p->volume_bounds.size[1] : 0.0f),
                       p->volume_bounds.origin[2] + ((k & 4) ? p->volume_bounds.size[2] : 0.0f), 1.0};
        double clip[4];
        for (int r = 0; r < 4; ++r) clip[r] = pv[r] * x[0] + pv[4 + r] * x[1] + pv[8 + r] * x[2] + pv[12 + r] * x[3];
        if (!(clip[3] > 1e-6) || !std::isfinite(clip[0] / clip[3]) || !std::isfinite(clip[1] / clip[3])) {
            rect[0] = rect[1] = 0; // a corner behind the camera (or the camera inside): the whole view
            rect[2] = p->width;
            rect[3] = p->height;
            return VKHR_OK;
        }
        for (int a = 0; a < 2; ++a) {
            lo[a] = std::min(lo[a], clip[a] / clip[3]);
            hi[a] = std::max(hi[a], clip[a] / clip[3]);
        }
    }
    // pixel centre (i + 0.5) / n * 2 - 1 in NDC; 2 pixels of margin for the FP32 ray set-up
    const double n[2] = {W, H};
    int64_t a0[2], a1[2];
    for (int a = 0; a < 2; ++a) {
        a0[a] = (int64_t)std::floor(std::max(-1e9, (lo[a] + 1.0) * 0.5 * n[a] - 0.5)) - 2;
        a1[a] = (int64_t)std::ceil(std::min(1e9, (hi[a] + 1.0) * 0.5 * n[a] - 0.5)) + 2;
        a0[a] = std::max<int64_t>(a0[a], 0);
        a1[a] = std::min<int64_t>(a1[a], (int64_t)n[a] - 1);
    }
    if (a0[0] > a1[0] || a0[1] > a1[1]) {
        rect[0] = rect[1] = rect[2] = rect[3] = 0;
        return VKHR_OK;
    }
    rect[0] = (int32_t)a0[0];
    rect[1] = (int32_t)a0[1];
    rect[2] = (int32_t)(a1[0] - a0[0] + 1);
    rect[3] = (int32_t)(a1[1] - a0[1] + 1);
    return VKHR_OK;
}

// ---- raymarch without allocations ---------------------------------------------------------
// For callers that may not allocate device memory at all: a real-time frame
// loop that forbids cudaMalloc (it synchronises the device and its latency is
// unbounded), or a host engine that owns the GPU memory budget and does not
// let plugins allocate.  The only scratch the raymarch needs, the brick
// occupancy bitmap, lives in a fixed array in the library's device image.
namespace {

constexpr size_t kStaticOccupancyWords = 32768; // 128 KiB: up to 1,048,576 occupancy bricks
constexpr int kMaxStaticDevices = 64;

__device__ __align__(256) uint32_t g_static_occupancy[kStaticOccupancyWords];

// Per device: the array's device address and the SM count, resolved by the
// first call on the device that succeeds (a failed lookup is retried).
std::mutex g_static_mutex;
bool g_static_resolved[kMaxStaticDevices];
uint32_t* g_static_occupancy_ptr[kMaxStaticDevices];
int g_static_sm_count[kMaxStaticDevices];

template <int DF, int TF>
cudaError_t launch_static(const RayConsts& c, const void* dens, const void* tang, const float* din, float* rgba,
                          float* dout, uint32_t* occ, size_t words, int sm_count, const int32_t rect[4], cudaStream_t st)
{
    // the array keeps the previous call's bits: clear the part this grid uses
    cudaError_t e = cudaMemsetAsync(occ, 0, words * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const typename DensityTexel<DF>::T* dd = (const typename DensityTexel<DF>::T*)dens;
    const int L = occupancy_lanes(c.res[0], c.res[1], c.res[2], sm_count);
    const unsigned ob = occupancy_blocks(c.res[0], c.res[1], c.res[2], sm_count, L);
    if (L == 8)
        occupancy_kernel<DF, 8><<<ob, 128, 0, st>>>(dd, c.res[0], c.res[1], c.res[2], c.nb[0], c.nb[1], c.nb[2], occ);
    else
        occupancy_kernel<DF, 1><<<ob, 128, 0, st>>>(dd, c.res[0], c.res[1], c.res[2], c.nb[0], c.nb[1], c.nb[2], occ);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int x0 = rect[0], y0 = rect[1], x1 = rect[0] + rect[2], y1 = rect[1] + rect[3];
    float4* out = reinterpret_cast<float4*>(rgba);
    if (rect[2] < c.W || rect[3] < c.H) {
        background_kernel<<<(unsigned)sm_count * 8, 256, 0, st>>>(out, dout, c.W, c.H, x0, y0, x1, y1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (rect[2] > 0 && rect[3] > 0) {
        const dim3 block(32 * kWarpsX * kWarpsY);
        const dim3 grid((rect[2] + kTileW * kWarpsX - 1) / (kTileW * kWarpsX),
                        (rect[3] + kTileH * kWarpsY - 1) / (kTileH * kWarpsY));
        raymarch_kernel<DF, TF><<<grid, block, 0, st>>>(c, (const typename DensityTexel<DF>::T*)dens, tang, occ, din,
                                                         out, dout, x0, y0, x1, y1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

} // namespace

extern "C" vkhr_status vkhr_raymarch_static(const vkhr_raymarch_params* params, const void* d_density,
                                            const void* d_tangent, const float* d_depth_in, float* d_rgba,
                                            float* d_depth_out, void* stream)
{
    if (!params || !d_density || !d_tangent || !d_rgba) return VKHR_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_rgba) & 15u) return VKHR_ERR_INVALID_ARG;
    const size_t tan_align = params->tangent_format == VKHR_TANGENT_I8_SNORM ? 4 : 16;
    if (reinterpret_cast<uintptr_t>(d_tangent) & (tan_align - 1)) return VKHR_ERR_INVALID_ARG;
    RayConsts c;
    vkhr_status s = make_consts(nullptr, params, c);
    if (s != VKHR_OK) return s;
    const size_t bricks = (size_t)c.nb[0] * c.nb[1] * c.nb[2];
    const size_t words = (bricks + 31) / 32;
    if (words > kStaticOccupancyWords) return VKHR_ERR_CAPACITY; // grid above the fixed scratch (~800^3)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return VKHR_ERR_CUDA;
    if (dev < 0 || dev >= kMaxStaticDevices) return VKHR_ERR_NOT_SUPPORTED;
    // first successful call on this device: resolve the array's device
    // address (host code cannot use the symbol itself) and the SM count
    {
        std::lock_guard<std::mutex> lock(g_static_mutex);
        if (!g_static_resolved[dev]) {
            uint32_t* ptr = nullptr;
            int sms = 0;
            cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_static_occupancy);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) {
                cudaGetLastError(); // leave no error of the failed lookup behind; a later call retries
                return VKHR_ERR_CUDA;
            }
            g_static_occupancy_ptr[dev] = ptr;
            g_static_sm_count[dev] = sms;
            g_static_resolved[dev] = true;
        }
    }
    int32_t rect[4]; // pixels outside it miss the volume's box
    if (vkhr_raymarch_footprint(params, rect) != VKHR_OK) return VKHR_ERR_INVALID_ARG;
    uint32_t* occ = g_static_occupancy_ptr[dev];
    const int sms = g_static_sm_count[dev];
    cudaStream_t st = (cudaStream_t)stream;
    const int df = params->density_format, tf = params->tangent_format;
    cudaError_t e;
    if (df == VKHR_DENSITY_U8_UNORM && tf == VKHR_TANGENT_I8_SNORM)
        e = launch_static<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_I8_SNORM>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    else if (df == VKHR_DENSITY_U8_UNORM)
        e = launch_static<VKHR_DENSITY_U8_UNORM, VKHR_TANGENT_F32X4>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    else if (df == VKHR_DENSITY_U32_COUNT && tf == VKHR_TANGENT_I8_SNORM)
        e = launch_static<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_I8_SNORM>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    else if (df == VKHR_DENSITY_U32_COUNT)
        e = launch_static<VKHR_DENSITY_U32_COUNT, VKHR_TANGENT_F32X4>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    else if (tf == VKHR_TANGENT_I8_SNORM)
        e = launch_static<VKHR_DENSITY_F32, VKHR_TANGENT_I8_SNORM>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    else
        e = launch_static<VKHR_DENSITY_F32, VKHR_TANGENT_F32X4>(c, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, occ, words, sms, rect, st);
    return e == cudaSuccess ? VKHR_OK : VKHR_ERR_CUDA;
}
