// march.cuh -- device code of the volume raymarch shared by the forward
// kernels (raymarch.cu) and the differentiable path (adjoint.cu): ray
// constants, texel formats and filtering, the occupancy bitmap, and the
// per-pixel march of share/shaders/volumes/volume.frag:31-103.
#pragma once
#include "common.cuh"

#include <algorithm>
#include <cmath>

namespace {


constexpr int kTileW = 8, kTileH = 4;         // pixels per warp
constexpr int kWarpsX = 2, kWarpsY = 2;       // warps per block
constexpr float kMaxSteps = 1048576.0f;       // 2^20: t += 1/steps still advances below 1
constexpr int kMaxAoDirections = 32;          // directional AO taps (vkhr_raymarch_params::ao_directions)

struct RayConsts {
    int W, H;
    float ray_dir[3][3][2];   // ray direction of pixel (px, py), up to a positive scale, as an unevaluated
                              // sum hi + lo per coefficient: component k = [k][0] + [k][1] px + [k][2] py
    float ray_w[3];           // homogeneous w of the unprojected far-plane point: w0 + wx px + wy py (its sign
                              // orients the direction)
    float pv[16];
    float cam[3];
    float radius;
    float lo[3], hi[3];
    int res[3];
    float tsc[3], tbias[3];   // texel coordinate u = P * tsc + tbias = (P - origin) / size * N - 0.5
    float voxel_space[3];
    float light[3], intensity[3], color[3];
    float alpha, exponent, iso, kd;
    float steps, shadow_steps, thickness, ao_kernel, ao_radius, ao_exp, ao_max;
    float lod;
    int shading_model, deep_shadows_on;
    int steps_pow2, shadow_pow2;  // 1/steps is exact and t = i * step: empty space may be jumped
    int nb[3];                    // occupancy bricks per axis, (res + 8) / 8
    float exponent2;              // second specular lobe's exponent (0: one lobe)
    float shift[2];               // tangent shift of each lobe (0: the reference's unshifted lobe)
    int ao_n;                     // directional AO taps (0: the ao_kernel^3 cube)
    float ao_off[kMaxAoDirections][3]; // world-space offsets of the directional taps
    unsigned long long tex;       // the density as a texture object (texture-unit and gather variants; else 0)
    int gshift;                   // gather variant: log2 of the slice tiles per row of its 2D texture
};

// Where the march's density samples come from: the texels in memory with the
// software trilinear below; the texture unit's hardware trilinear filter,
// whose weights have 8 fractional bits -- for every sample (kSampleTexture),
// or for the shadow and ambient-occlusion samples of the shading only while
// the isosurface search reads memory (kSampleShadeTexture); or the texture
// unit's 2x2 gathers of exact texel values, which the software trilinear
// then filters (kSampleGather: the memory path's pixels, bit for bit).
constexpr int kSampleMemory = 0, kSampleTexture = 1, kSampleShadeTexture = 2, kSampleGather = 3;
__host__ __device__ constexpr int march_source(int src)
{
    return src == kSampleTexture || src == kSampleGather ? src : kSampleMemory;
}
__host__ __device__ constexpr int shade_source(int src)
{
    return src == kSampleMemory || src == kSampleGather ? src : kSampleTexture;
}

constexpr int kBrick = 8;          // occupancy brick edge in texel cells
constexpr float kSkipMargin = 0.01f; // texels kept between a predicted sample and a brick face

template <int DF>
struct DensityTexel;
template <>
struct DensityTexel<VKHR_DENSITY_U8_UNORM> {
    typedef uint8_t T;
    static __device__ __forceinline__ float load(const T* p, size_t i) { return (float)__ldg(p + i); }
    static constexpr float scale = 1.0f / 255.0f; // UNORM c / 255
};
template <>
struct DensityTexel<VKHR_DENSITY_U32_COUNT> {
    typedef uint32_t T;
    static __device__ __forceinline__ float load(const T* p, size_t i) { return (float)__ldg(p + i); }
    static constexpr float scale = 1.0f;
};
template <>
struct DensityTexel<VKHR_DENSITY_F32> {
    typedef float T;
    static __device__ __forceinline__ float load(const T* p, size_t i) { return __ldg(p + i); }
    static constexpr float scale = 1.0f;
};

struct Vec3 {
    float x, y, z;
};
__device__ __forceinline__ Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
__device__ __forceinline__ Vec3 operator+(Vec3 a, Vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ Vec3 operator-(Vec3 a, Vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ Vec3 operator*(Vec3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ Vec3 normalize(Vec3 a)
{
    float l = sqrtf(dot(a, a));
    return v3(a.x / l, a.y / l, a.z / l); // 0/0 -> NaN for a zero vector, as on the GPU
}
// GLSL mix(x, y, a) = x * (1 - a) + y * a
__device__ __forceinline__ Vec3 mix(Vec3 a, Vec3 b, float t)
{
    const float u = 1.0f - t;
    return v3(fmaf(b.x, t, a.x * u), fmaf(b.y, t, a.y * u), fmaf(b.z, t, a.z * u));
}
__device__ __forceinline__ float clip_depth(const RayConsts& c, Vec3 p)
{
    float z = fmaf(c.pv[2], p.x, fmaf(c.pv[6], p.y, fmaf(c.pv[10], p.z, c.pv[14])));
    float w = fmaf(c.pv[3], p.x, fmaf(c.pv[7], p.y, fmaf(c.pv[11], p.z, c.pv[15])));
    return z / w;
}

// Texel-space set-up; false when all eight taps read the border.
__device__ __forceinline__ bool tex_setup(const RayConsts& c, Vec3 p, int i0[3], float a[3])
{
    const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float u = fmaf(pp[k], c.tsc[k], c.tbias[k]);
        if (!(u > -2.0f && u < (float)(c.res[k] + 1))) return false;
        float f = floorf(u);
        i0[k] = (int)f;
        a[k] = u - f;
    }
    return true;
}

// The reference sampler's filter of the eight taps v (x fastest, then y, then z)
// at fractions a.
__device__ __forceinline__ float trilinear(const float v[8], const float a[3])
{
    const float x00 = fmaf(a[0], v[1] - v[0], v[0]);
    const float x10 = fmaf(a[0], v[3] - v[2], v[2]);
    const float x01 = fmaf(a[0], v[5] - v[4], v[4]);
    const float x11 = fmaf(a[0], v[7] - v[6], v[6]);
    const float y0 = fmaf(a[1], x10 - x00, x00);
    const float y1 = fmaf(a[1], x11 - x01, x01);
    return fmaf(a[2], y1 - y0, y0);
}

template <int DF>
__device__ __forceinline__ float sample_density(const RayConsts& c, const typename DensityTexel<DF>::T* __restrict__ d,
                                                Vec3 p)
{
    typedef DensityTexel<DF> TX;
    int i0[3];
    float a[3];
    if (!tex_setup(c, p, i0, a)) return 0.0f;
    const int nx = c.res[0], ny = c.res[1], nz = c.res[2];
    float v[8];
    if (i0[0] >= 0 && i0[0] + 1 < nx && i0[1] >= 0 && i0[1] + 1 < ny && i0[2] >= 0 && i0[2] + 1 < nz) {
        const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
        const size_t b = (size_t)i0[0] + sy * i0[1] + sz * i0[2];
        v[0] = TX::load(d, b);
        v[1] = TX::load(d, b + 1);
        v[2] = TX::load(d, b + sy);
        v[3] = TX::load(d, b + sy + 1);
        v[4] = TX::load(d, b + sz);
        v[5] = TX::load(d, b + sz + 1);
        v[6] = TX::load(d, b + sz + sy);
        v[7] = TX::load(d, b + sz + sy + 1);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int x = i0[0] + (k & 1), y = i0[1] + ((k >> 1) & 1), z = i0[2] + (k >> 2);
            v[k] = (x >= 0 && y >= 0 && z >= 0 && x < nx && y < ny && z < nz)
                       ? TX::load(d, (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z))
                       : 0.0f;
        }
    }
    return trilinear(v, a) * TX::scale;
}

// The 2x2 texels of a gather as floats: element-type reads, so each value is
// the texel's own (u8 and u32 converted exactly as the memory path does).
template <int DF>
struct GatherTexel;
template <>
struct GatherTexel<VKHR_DENSITY_U8_UNORM> {
    static __device__ __forceinline__ float4 get(unsigned long long t, float x, float y)
    {
        const uchar4 g = tex2Dgather<uchar4>((cudaTextureObject_t)t, x, y, 0);
        return make_float4((float)g.x, (float)g.y, (float)g.z, (float)g.w);
    }
};
template <>
struct GatherTexel<VKHR_DENSITY_U32_COUNT> {
    static __device__ __forceinline__ float4 get(unsigned long long t, float x, float y)
    {
        const uint4 g = tex2Dgather<uint4>((cudaTextureObject_t)t, x, y, 0);
        return make_float4((float)g.x, (float)g.y, (float)g.z, (float)g.w);
    }
};
template <>
struct GatherTexel<VKHR_DENSITY_F32> {
    static __device__ __forceinline__ float4 get(unsigned long long t, float x, float y)
    {
        return tex2Dgather<float4>((cudaTextureObject_t)t, x, y, 0);
    }
};

// sample_density through the texture unit's gathers.  The density is a 2D
// texture of the grid's z slices, tiled 2^gshift per row, each slice framed
// by a one-texel border of zeros (tiles of (w + 2) x (h + 2)); texel (x, y)
// of slice z sits at column (z mod 2^gshift) (w + 2) + 1 + x and row
// (z >> gshift) (h + 2) + 1 + y.  One gather per slice returns the four
// texels (x0..x0+1, y0..y0+1) -- the frames and the texture's border give
// the zeros outside the grid -- in the order (x0, y1), (x1, y1), (x1, y0),
// (x0, y0); the software trilinear filters them as sample_density does.
template <int DF>
__device__ __forceinline__ float sample_density_gather(const RayConsts& c, Vec3 p)
{
    typedef DensityTexel<DF> TX;
    int i0[3];
    float a[3];
    if (!tex_setup(c, p, i0, a)) return 0.0f;
    const int tw = c.res[0] + 2, th = c.res[1] + 2, mask = (1 << c.gshift) - 1;
    float v[8];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz) {
        const int z = i0[2] + dz;
        float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (z >= 0 && z < c.res[2]) // coordinates between the two columns / rows: exact integers + 1
            g = GatherTexel<DF>::get(c.tex, (float)((z & mask) * tw + i0[0] + 2),
                                     (float)((z >> c.gshift) * th + i0[1] + 2));
        v[4 * dz + 0] = g.w;
        v[4 * dz + 1] = g.z;
        v[4 * dz + 2] = g.x;
        v[4 * dz + 3] = g.y;
    }
    return trilinear(v, a) * TX::scale;
}

template <int DF, int SRC>
__device__ __forceinline__ float density_at(const RayConsts& c, const typename DensityTexel<DF>::T* __restrict__ d,
                                            Vec3 p)
{
    if (SRC == kSampleGather) return sample_density_gather<DF>(c, p);
    if (SRC == kSampleTexture) { // texel centres at integer + 0.5 in the texture's unnormalised coordinates
        const float u = fmaf(p.x, c.tsc[0], c.tbias[0]), v = fmaf(p.y, c.tsc[1], c.tbias[1]),
                    w = fmaf(p.z, c.tsc[2], c.tbias[2]);
        return tex3D<float>((cudaTextureObject_t)c.tex, u + 0.5f, v + 0.5f, w + 0.5f);
    }
    return sample_density<DF>(c, d, p);
}

template <int TF>
__device__ __forceinline__ Vec3 tangent_texel(const void* t, int x, int y, int z, const int* n)
{
    if (x < 0 || y < 0 || z < 0 || x >= n[0] || y >= n[1] || z >= n[2]) return v3(0.0f, 0.0f, 0.0f);
    const size_t i = (size_t)x + (size_t)n[0] * ((size_t)y + (size_t)n[1] * z);
    if (TF == VKHR_TANGENT_I8_SNORM) {
        const char4 q = __ldg(reinterpret_cast<const char4*>(t) + i);
        return v3(fmaxf((float)q.x / 127.0f, -1.0f), fmaxf((float)q.y / 127.0f, -1.0f),
                  fmaxf((float)q.z / 127.0f, -1.0f));
    }
    const float4 f = __ldg(reinterpret_cast<const float4*>(t) + i);
    return v3(f.x, f.y, f.z);
}

template <int TF>
__device__ Vec3 sample_tangent(const RayConsts& c, const void* t, Vec3 p)
{
    int i0[3];
    float a[3];
    Vec3 acc = v3(0.0f, 0.0f, 0.0f);
    if (!tex_setup(c, p, i0, a)) return acc;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        const float w = (dx ? a[0] : 1.0f - a[0]) * (dy ? a[1] : 1.0f - a[1]) * (dz ? a[2] : 1.0f - a[2]);
        acc = acc + tangent_texel<TF>(t, i0[0] + dx, i0[1] + dy, i0[2] + dz, c.res) * w;
    }
    return acc;
}

// Occupancy of the texel-cell grid.  A sample with lower tap i0 = floor(u)
// (u = s * N - 0.5 per axis) reads texels i0 and i0 + 1; shifting to
// cell = i0 + 1 in [0, N], brick k covers cells [8k, 8k + 8), i.e. texels
// [8k - 1, 8k + 7].  A brick is occupied when any of those texels is nonzero;
// every sample whose cell lies in an empty brick is exactly 0.
//
// A column: the chunk of 8 texels along x at x0 = 8 * cx (one vector load
// when aligned) in each of the 8 x 8 rows y in [8a, 8a + 8), z in [8c, 8c + 8).
// Texel x0 + i belongs to cell brick cx (i <= 7) and texel x0 + 7 also to
// cx + 1; along y (and z) row 8a + i belongs to cell brick a, and row 8a + 7
// also to a + 1.  The column's rows' masks are ORed (in registers and across
// its 8 lanes) and it marks at most 8 bricks.
template <int DF>
__device__ __forceinline__ uint32_t chunk_mask(const typename DensityTexel<DF>::T* __restrict__ p, int n)
{
    typedef DensityTexel<DF> TX;
    uint32_t m = 0;
    if (n == 8 && DF == VKHR_DENSITY_U8_UNORM && !(reinterpret_cast<uintptr_t>(p) & 7u)) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            m |= ((v.x >> (8 * i)) & 0xffu) ? (1u << i) : 0u;
            m |= ((v.y >> (8 * i)) & 0xffu) ? (1u << (i + 4)) : 0u;
        }
    } else if (n == 8 && DF != VKHR_DENSITY_U8_UNORM && !(reinterpret_cast<uintptr_t>(p) & 15u)) {
        const float4* q = reinterpret_cast<const float4*>(p);
        const float4 a = __ldg(q), b = __ldg(q + 1);
        const float f[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        const uint32_t* w = reinterpret_cast<const uint32_t*>(f);
#pragma unroll
        for (int i = 0; i < 8; ++i) // u32 counts: nonzero bits; f32: nonzero value (-0 is zero)
            m |= (DF == VKHR_DENSITY_F32 ? f[i] != 0.0f : w[i] != 0u) ? (1u << i) : 0u;
    } else {
        for (int i = 0; i < n; ++i) m |= TX::load(p, i) != 0.0f ? (1u << i) : 0u;
    }
    return m;
}

__device__ __forceinline__ void occupancy_mark(uint32_t* bits, int nbx, int nby, int kx, int ky, int kz)
{
    const uint32_t b = (uint32_t)kx + (uint32_t)nbx * ((uint32_t)ky + (uint32_t)nby * (uint32_t)kz);
    atomicOr(bits + (b >> 5), 1u << (b & 31)); // result unused: a fire-and-forget reduction
}

// One 8x8x8 column of texels (chunk cx of rows 8a..8a+7 of planes 8c..8c+7)
// with L lanes (L = 1 or 8): lane sub = lane % L reads the z rows
// zz = sub, sub + L, ...; the masks are ORed across the column's L lanes by
// shuffles (only the lane holding zz = 7 contributes the last-plane masks)
// and lane sub = 0 marks.  With L > 1 all 32 lanes of the warp call it
// (valid = false for lanes past the last column); for a given zz the warp's
// 32 / L columns read consecutive chunks of one row.
template <int DF, int L>
__device__ __forceinline__ void occupancy_column(const typename DensityTexel<DF>::T* __restrict__ d, int nx, int ny,
                                                 int nz, int nbx, int nby, uint32_t* bits, int cx, int a, int c,
                                                 bool valid)
{
    const int sub = (int)(threadIdx.x & 31u) & (L - 1);
    uint32_t m_all = 0, m_y = 0, m_z = 0, m_yz = 0; // rows of brick (a, c); last y row; last z row; both
    if (valid) {
        const int x0 = 8 * cx, n = min(8, nx - x0);
#pragma unroll
        for (int k = 0; k < 8 / L; ++k) {
            const int zz = sub + k * L, z = 8 * c + zz;
            if (z >= nz) break;
            uint32_t mz = 0, my = 0;
#pragma unroll
            for (int yy = 0; yy < 8; ++yy) {
                const int y = 8 * a + yy;
                if (y < ny) {
                    const uint32_t m = chunk_mask<DF>(d + (size_t)nx * ((size_t)y + (size_t)ny * z) + x0, n);
                    mz |= m;
                    if (yy == 7) my = m;
                }
            }
            m_all |= mz;
            m_y |= my;
            if (zz == 7) {
                m_z = mz;
                m_yz = my;
            }
        }
    }
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
        m_all |= __shfl_xor_sync(0xffffffffu, m_all, o);
        m_y |= __shfl_xor_sync(0xffffffffu, m_y, o);
        m_z |= __shfl_xor_sync(0xffffffffu, m_z, o);
        m_yz |= __shfl_xor_sync(0xffffffffu, m_yz, o);
    }
    if (!valid || sub != 0) return;
    const uint32_t ms[4] = {m_all, m_y, m_z, m_yz};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!ms[k]) continue;
        const int ky = a + (k & 1), kz = c + (k >> 1);
        occupancy_mark(bits, nbx, nby, cx, ky, kz);
        if (ms[k] & 0x80u) occupancy_mark(bits, nbx, nby, cx + 1, ky, kz);
    }
}

template <int DF, int L>
__global__ void occupancy_kernel(const typename DensityTexel<DF>::T* __restrict__ d, int nx, int ny, int nz, int bx,
                                 int by, int bz, uint32_t* __restrict__ bits)
{
    // L lanes per column, columns with cx fastest; the loop is warp-uniform
    const uint32_t cxn = (uint32_t)(nx + 7) / 8, an = (uint32_t)(ny + 7) / 8, cn = (uint32_t)(nz + 7) / 8;
    const uint64_t lanes = (uint64_t)L * cxn * an * cn;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g - (threadIdx.x & 31u) < lanes; g += stride) {
        const bool valid = g < lanes;
        const uint32_t i = valid ? (uint32_t)(g / L) : 0u;
        const uint32_t r = i / cxn, cx = i - r * cxn;
        const uint32_t c = r / an, a = r - c * an;
        occupancy_column<DF, L>(d, nx, ny, nz, bx, by, bits, (int)cx, (int)a, (int)c, valid);
    }
}

static inline uint64_t occupancy_columns(int nx, int ny, int nz)
{
    return (uint64_t)((nx + 7) / 8) * ((ny + 7) / 8) * ((nz + 7) / 8);
}

// Lanes per column: 8 when that grid still fits in 16 blocks of 128 threads
// per SM (a small volume has too few columns to fill the GPU one per
// thread), else 1.
static inline int occupancy_lanes(int nx, int ny, int nz, int sm_count)
{
    return 8 * occupancy_columns(nx, ny, nz) <= (uint64_t)sm_count * 16 * 128 ? 8 : 1;
}

static inline unsigned occupancy_blocks(int nx, int ny, int nz, int sm_count, int lanes_per_column)
{
    const uint64_t lanes = (uint64_t)lanes_per_column * occupancy_columns(nx, ny, nz);
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((lanes + 127) / 128, (uint64_t)sm_count * 16));
}

// The occupancy brick of a sample's texel cell (cell = floor(u) + 1 per axis,
// in [0, N]; classify's index), for a sample inside the cell grid.
__device__ __forceinline__ uint32_t cell_brick(const RayConsts& c, const float u[3])
{
    const int bxk = ((int)floorf(u[0]) + 1) / kBrick, byk = ((int)floorf(u[1]) + 1) / kBrick,
              bzk = ((int)floorf(u[2]) + 1) / kBrick;
    return (uint32_t)bxk + (uint32_t)c.nb[0] * ((uint32_t)byk + (uint32_t)c.nb[1] * (uint32_t)bzk);
}

// Classifies one sample position (texel coordinates u).  Returns 1 when the
// sample is exactly zero (border, or an empty brick), 2 when it is zero and
// the ray has left the grid for good (moving away along every such axis),
// 0 when it must be sampled.  box_lo/box_hi receive the current brick's
// texel-coordinate extent for the empty-space jump.  du only needs the ray
// direction's sign per axis (its reciprocal serves).
__device__ __forceinline__ int classify(const RayConsts& c, const uint32_t* __restrict__ occ, const float u[3],
                                        const float du[3], float box_lo[3], float box_hi[3])
{
    int cell[3];
    bool outside = false, leaving = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float f = floorf(u[k]);
        if (!(f >= -1.0f && f <= (float)(c.res[k] - 1))) {
            outside = true;
            if ((u[k] < -1.0f - kSkipMargin && du[k] <= 0.0f) || (u[k] > (float)c.res[k] + kSkipMargin && du[k] >= 0.0f) ||
                !(u[k] == u[k]))
                leaving = true;
            cell[k] = 0;
        } else {
            cell[k] = (int)f + 1;
        }
    }
    if (outside) { // zero, but no brick to jump across: step singly
#pragma unroll
        for (int k = 0; k < 3; ++k) box_lo[k] = box_hi[k] = u[k];
        return leaving ? 2 : 1;
    }
    const int bxk = cell[0] / kBrick, byk = cell[1] / kBrick, bzk = cell[2] / kBrick;
    const uint32_t b = (uint32_t)bxk + (uint32_t)c.nb[0] * ((uint32_t)byk + (uint32_t)c.nb[1] * (uint32_t)bzk);
    if (__ldg(occ + (b >> 5)) & (1u << (b & 31))) return 0;
    box_lo[0] = (float)(kBrick * bxk - 1);
    box_lo[1] = (float)(kBrick * byk - 1);
    box_lo[2] = (float)(kBrick * bzk - 1);
    box_hi[0] = box_lo[0] + (float)kBrick;
    box_hi[1] = box_lo[1] + (float)kBrick;
    box_hi[2] = box_lo[2] + (float)kBrick;
    return 1;
}

// Whole steps that stay inside the empty brick [lo, hi) from u along du
// (per unit t), keeping kSkipMargin texels from its faces.  inv holds 1/du
// per axis (0 where du is 0; computed once per ray, and it carries du's
// sign, which is all classify needs) and steps_per_t = 1/step, exact because
// jumps run for power-of-two step counts only.  The reciprocal's rounding
// moves the predicted exit by about 1e-6 texel, far inside the margin; and
// even one step more than the exact count would leave every skipped sample
// inside the margin-shrunk brick (the first sample past the jump is taken).
__device__ __forceinline__ float steps_inside(const float u[3], const float inv[3], const float lo[3], const float hi[3],
                                              float steps_per_t)
{
    float te = INFINITY;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (inv[k] > 0.0f) te = fminf(te, (hi[k] - kSkipMargin - u[k]) * inv[k]);
        else if (inv[k] < 0.0f) te = fminf(te, (lo[k] + kSkipMargin - u[k]) * inv[k]);
    }
    return floorf(te * steps_per_t);
}

__device__ __forceinline__ void reciprocals(const float d[3], float inv[3])
{
#pragma unroll
    for (int k = 0; k < 3; ++k) inv[k] = d[k] != 0.0f ? 1.0f / d[k] : 0.0f;
}

__device__ __forceinline__ void texel_coords(const RayConsts& c, Vec3 p, float u[3])
{
    u[0] = fmaf(p.x, c.tsc[0], c.tbias[0]);
    u[1] = fmaf(p.y, c.tsc[1], c.tbias[1]);
    u[2] = fmaf(p.z, c.tsc[2], c.tbias[2]);
}

// Tangent of a Kajiya-Kay lobe shifted by s towards the camera,
// normalize(T + s N) with N the unit component of -E perpendicular to T,
// as its cosines with L and E: with a = T.L, b = T.E, c = L.E, sb = sin(T, E)
// and k = 1 / sqrt(1 + s^2),
//   a_s = k (a + s (a b - c) / sb),   b_s = k (b - s sb)
// (T itself where N is undefined, sb = 0).  s = 0 leaves a and b unchanged.
__device__ __forceinline__ void shift_cosines(float a, float b, float sb, float cab, float s, float& as, float& bs)
{
    as = a;
    bs = b;
    if (s != 0.0f && sb > 0.0f) {
        const float k = 1.0f / sqrtf(fmaf(s, s, 1.0f));
        as = k * (a + s * (a * b - cab) / sb);
        bs = k * (b - s * sb);
    }
}

// One Kajiya-Kay specular lobe (kajiya-kay.glsl:15-21) of the tangent
// shifted by s: max(cos(T_s,L) cos(T_s,E) + sin(T_s,L) sin(T_s,E), 0)^p.  For
// s = 0 it is the reference's expression of the unshifted cosines and sines.
__device__ __forceinline__ float kk_lobe(float cosTL, float cosTE, float sinTL, float sinTE, float cosLE, float s,
                                         float p)
{
    if (s == 0.0f) return powf(fmaxf(cosTL * cosTE + sinTL * sinTE, 0.0f), p);
    float a, b;
    shift_cosines(cosTL, cosTE, sinTE, cosLE, s, a, b);
    const float sa = sqrtf(fmaxf(1.0f - a * a, 0.0f)), sb = sqrtf(fmaxf(1.0f - b * b, 0.0f));
    return powf(fmaxf(a * b + sa * sb, 0.0f), p);
}

// What the differentiable path keeps of a pixel's forward march (32 bytes).
struct PixelTape {
    float surf[3];   // surface point
    float acc;       // accumulated density of the primary march
    float occl_s;    // (1 - alpha)^strands of the density shadows (1 when off)
    float dsum;      // LAO sum of min(density, ao_max) (0 when off)
    uint32_t n;      // primary-march iterations taken (skipped zero samples included)
    uint32_t flags;  // kTapeEmitted | kTapeHit
};
constexpr uint32_t kTapeEmitted = 1u, kTapeHit = 2u;

// Double-float arithmetic: a value as an unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi) / 2), with error-free FMA products and two-sums
// (T. J. Dekker, "A floating-point technique for extending the available
// precision", 1971; the FMA form of the product).  The intrinsics keep the
// compiler from contracting the steps whose rounding errors they capture.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_fast_sum(float a, float b) // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_add(DF x, DF y)
{
    const DF s = df_two_sum(x.hi, y.hi);
    return df_fast_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ DF df_mul_f(DF x, float f)
{
    const float p = __fmul_rn(x.hi, f);
    return df_fast_sum(p, __fmaf_rn(x.lo, f, __fmaf_rn(x.hi, f, -p)));
}
__device__ __forceinline__ DF df_mul(DF x, DF y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    return df_fast_sum(p, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.hi, -p))));
}
__device__ __forceinline__ DF df_div(DF n, DF d)
{
    const float q1 = __fdiv_rn(n.hi, d.hi);
    const DF r = df_add(n, df_mul_f(d, -q1)); // n - q1 d
    return df_fast_sum(q1, __fdiv_rn(r.hi, d.hi));
}

// Entry of the pixel-centre ray into the volume's AABB (the front faces of
// the proxy cube, volume.vert:17-25), and the march's end point
// start + normalize(start - camera) * radius (volume.frag:32-34).  The ray
// points from the camera at the pixel's far-plane point, inverse(P V)
// (nx, ny, 1, 1) dehomogenised.  That point's w is about 1/far, the
// difference of nearly equal terms, so the direction is taken as
// num - camera * w (num the xyz of the unprojection): the same ray up to the
// positive factor w, affine in the pixel's integer coordinates, with
// coefficients folded in double on the host and kept as float pairs.  The
// direction and the entry on the hit face are evaluated in double-float:
// for a camera tens of units away, FP32 alone would place the entry a few
// 1e-5 texel off, enough to flip the shader's isosurface and zero tests.
__device__ __forceinline__ bool ray_entry(const RayConsts& c, int px, int py, Vec3& start, Vec3& end)
{
    const float fx = (float)px, fy = (float)py; // exact
    const float w = fmaf(c.ray_w[1], fx, fmaf(c.ray_w[2], fy, c.ray_w[0]));
    DF D[3];
    float dir[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const DF a = DF{c.ray_dir[k][0][0], c.ray_dir[k][0][1]};
        const DF b = df_mul_f(DF{c.ray_dir[k][1][0], c.ray_dir[k][1][1]}, fx);
        const DF e = df_mul_f(DF{c.ray_dir[k][2][0], c.ray_dir[k][2][1]}, fy);
        D[k] = df_add(df_add(a, b), e);
        if (w < 0.0f) D[k] = DF{-D[k].hi, -D[k].lo}; // a far-plane point behind the camera flips the ray
        dir[k] = D[k].hi;
    }
    float tmin = -INFINITY, tmax = INFINITY;
    bool hit = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (dir[k] == 0.0f) {
            if (c.cam[k] < c.lo[k] || c.cam[k] > c.hi[k]) hit = false;
            continue;
        }
        float t0 = (c.lo[k] - c.cam[k]) / dir[k], t1 = (c.hi[k] - c.cam[k]) / dir[k];
        tmin = fmaxf(tmin, fminf(t0, t1));
        tmax = fminf(tmax, fmaxf(t0, t1));
    }
    if (!(hit && tmin > 0.0f && tmin <= tmax)) return false;
    // the entry on the face of the axis whose slab is entered last, in double-float
    int ke = 0;
    float best = -INFINITY;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (dir[k] == 0.0f) continue;
        const float near = fminf((c.lo[k] - c.cam[k]) / dir[k], (c.hi[k] - c.cam[k]) / dir[k]);
        if (near > best) {
            best = near;
            ke = k;
        }
    }
    const float face = dir[ke] > 0.0f ? c.lo[ke] : c.hi[ke];
    const DF t = df_div(df_two_sum(face, -c.cam[ke]), D[ke]);
    float p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const DF q = df_add(df_mul(t, D[k]), DF{c.cam[k], 0.0f});
        p[k] = k == ke ? face : __fadd_rn(q.hi, q.lo);
    }
    const Vec3 cam = v3(c.cam[0], c.cam[1], c.cam[2]);
    start = v3(p[0], p[1], p[2]);
    end = start + normalize(start - cam) * c.radius;
    return true;
}

// Ray groups: G lanes (a power of two, G <= 8) march one pixel's ray.  The
// lanes evaluate G consecutive samples at once (classification, the empty-
// space jump length, the density), then every lane replays the G outcomes
// in order -- the serial loop's decisions and sums in the serial order, so
// the pixel is the one-lane march's bit for bit -- and the group goes on
// from where the replay stopped or jumped.  A ray's chain of dependent L2
// loads gets up to G times shorter; the shadow march and the ambient-
// occlusion taps are split the same way.  Every branch the lanes of a group
// take is decided on values they share, so the group stays converged.
template <int G>
__device__ __forceinline__ unsigned group_mask()
{
    static_assert(G >= 2 && G <= 8 && (G & (G - 1)) == 0, "ray groups of 2, 4 or 8 lanes");
    return ((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
}

// The outcome of one sample of a march: 0 sampled (val = density), 1 exactly
// zero (val = the empty-space jump in steps, < 1: none), 2 left the grid, 3
// behind the depth buffer, 4 past the end of the march.
template <int G>
__device__ __forceinline__ void group_outcomes(int code, float val, int (&cs)[G], float (&vs)[G])
{
    const unsigned gm = group_mask<G>();
#pragma unroll
    for (int j = 0; j < G; ++j) {
        cs[j] = __shfl_sync(gm, code, j, G);
        vs[j] = __shfl_sync(gm, val, j, G);
    }
}

// The t of this lane's sample: `rank` plain steps past t, added one at a
// time as the serial loop adds them.
__device__ __forceinline__ float group_t(float t, float step, int rank)
{
    for (int i = 0; i < rank; ++i) t += step;
    return t;
}

// The fragment of a ray whose primary march ended with accumulated density
// acc and surface point surf (volume.frag:45-103): shading, density shadows,
// ambient occlusion, coverage and depth.  Leaves out / out_depth (background)
// alone when acc is 0 (the shader's discard).
template <int DF, int TF, bool TAPE = false, int SRC = kSampleMemory, int G = 1>
__device__ __forceinline__ void shade_fragment(const RayConsts& c, const typename DensityTexel<DF>::T* __restrict__ dens,
                                               const void* __restrict__ tang, const uint32_t* __restrict__ occ,
                                               Vec3 surf, float acc, float4& out, float& out_depth,
                                               PixelTape* tape = nullptr)
{
    const Vec3 cam = v3(c.cam[0], c.cam[1], c.cam[2]);
    const float a = acc / c.iso;
    if (a != 0.0f) {
        if (TAPE) tape->flags |= kTapeEmitted;
        const float coverage = c.lod * a * c.alpha;
        // ---- shading (volume.frag:50-67, kajiya-kay.glsl:7-24) ------------
        Vec3 shading = v3(1.0f, 1.0f, 1.0f);
        const Vec3 light = v3(c.light[0], c.light[1], c.light[2]);
        if (c.shading_model == VKHR_SHADING_KAJIYA_KAY) {
            const Vec3 L = normalize(light - surf);
            const Vec3 E = normalize(surf - cam);
            const Vec3 T = normalize(sample_tangent<TF>(c, tang, surf));
            const float cosTL = dot(T, L), cosTE = dot(T, E);
            const float sinTL = sqrtf(fmaxf(1.0f - cosTL * cosTL, 0.0f));
            const float sinTE = sqrtf(fmaxf(1.0f - cosTE * cosTE, 0.0f));
            const float cosLE = c.shift[0] != 0.0f || c.exponent2 > 0.0f ? dot(L, E) : 0.0f;
            const float spec = kk_lobe(cosTL, cosTE, sinTL, sinTE, cosLE, c.shift[0], c.exponent);
            const float dk = c.kd * sinTL;
            shading = v3(c.color[0] * dk + c.intensity[0] * spec, c.color[1] * dk + c.intensity[1] * spec,
                         c.color[2] * dk + c.intensity[2] * spec);
            if (c.exponent2 > 0.0f) { // the second, hair-coloured lobe
                const float spec2 = kk_lobe(cosTL, cosTE, sinTL, sinTE, cosLE, c.shift[1], c.exponent2);
                shading = shading + v3(c.intensity[0] * c.color[0] * spec2, c.intensity[1] * c.color[1] * spec2,
                                       c.intensity[2] * c.color[2] * spec2);
            }
        }
        float occlusion = 1.0f;
        // ---- volume_approximated_deep_shadows (approximate_deep_shadows.glsl:24-36)
        if (c.deep_shadows_on == 1 && c.shading_model != VKHR_SHADING_LAO) {
            const float sstep = 1.0f / c.shadow_steps;
            float ls[3], le[3], dl[3];
            texel_coords(c, surf, ls);
            texel_coords(c, light, le);
            dl[0] = le[0] - ls[0];
            dl[1] = le[1] - ls[1];
            dl[2] = le[2] - ls[2];
            float inv_dl[3];
            reciprocals(dl, inv_dl);
            float strands = 0.0f;
            if constexpr (G == 1) {
                for (float t = 0.0f; t < 1.0f;) {
                    const Vec3 Q = mix(surf, light, t);
                    float u[3], lo[3], hi[3];
                    texel_coords(c, Q, u);
                    const int z = classify(c, occ, u, inv_dl, lo, hi);
                    if (z == 2) break;
                    if (z == 1) {
                        const float n = c.shadow_pow2 ? steps_inside(u, inv_dl, lo, hi, c.shadow_steps) : 0.0f;
                        t = n >= 1.0f ? fmaf(n, sstep, t) : t + sstep;
                        continue;
                    }
                    strands += density_at<DF, shade_source(SRC)>(c, dens, Q) * c.thickness;
                    t += sstep;
                }
            } else { // the same samples and sum, G at a time
                const int rank = (int)(threadIdx.x & (G - 1));
                for (float t = 0.0f; t < 1.0f;) {
                    const float tr = group_t(t, sstep, rank);
                    int code = 4;
                    float val = 0.0f;
                    if (tr < 1.0f) {
                        const Vec3 Q = mix(surf, light, tr);
                        float u[3], lo[3], hi[3];
                        texel_coords(c, Q, u);
                        code = classify(c, occ, u, inv_dl, lo, hi);
                        if (code == 1) val = c.shadow_pow2 ? steps_inside(u, inv_dl, lo, hi, c.shadow_steps) : 0.0f;
                        else if (code == 0) val = density_at<DF, shade_source(SRC)>(c, dens, Q);
                    }
                    int cs[G];
                    float vs[G];
                    group_outcomes<G>(code, val, cs, vs);
                    bool stop = false, jumped = false;
                    float tc = t;
#pragma unroll
                    for (int j = 0; j < G; ++j) {
                        if (stop || jumped) continue;
                        if (cs[j] >= 2) {
                            stop = true;
                        } else if (cs[j] == 1 && vs[j] >= 1.0f) {
                            t = fmaf(vs[j], sstep, tc);
                            jumped = true;
                        } else {
                            if (cs[j] == 0) strands += vs[j] * c.thickness;
                            tc += sstep;
                        }
                    }
                    if (stop) break;
                    if (!jumped) t = tc;
                }
            }
            const float os = powf(1.0f - c.alpha, strands);
            if (TAPE) tape->occl_s = os;
            occlusion *= os;
        }
        // ---- local_ambient_occlusion (local_ambient_occlusion.glsl:9-30)
        if (c.shading_model != VKHR_SHADING_ADSM) {
            float dsum = 0.0f, taps;
            if (c.ao_n > 0) { // the directional extension
                if constexpr (G == 1) {
                    for (int i = 0; i < c.ao_n; ++i) {
                        const Vec3 q = v3(surf.x + c.ao_off[i][0], surf.y + c.ao_off[i][1], surf.z + c.ao_off[i][2]);
                        dsum += fminf(density_at<DF, shade_source(SRC)>(c, dens, q), c.ao_max);
                    }
                } else { // G taps at a time, added in tap order
                    const int rank = (int)(threadIdx.x & (G - 1));
                    for (int base = 0; base < c.ao_n; base += G) {
                        const int i = base + rank;
                        float d = 0.0f;
                        if (i < c.ao_n) {
                            const Vec3 q = v3(surf.x + c.ao_off[i][0], surf.y + c.ao_off[i][1], surf.z + c.ao_off[i][2]);
                            d = density_at<DF, shade_source(SRC)>(c, dens, q);
                        }
                        int cs[G];
                        float vs[G];
                        group_outcomes<G>(0, d, cs, vs);
#pragma unroll
                        for (int j = 0; j < G; ++j)
                            if (base + j < c.ao_n) dsum += fminf(vs[j], c.ao_max);
                    }
                }
                taps = (float)c.ao_n;
            } else {
                const float kr = (c.ao_kernel - 1.0f) / 2.0f;
                const float scale = c.ao_radius / kr;
                const Vec3 sc = v3(c.voxel_space[0] * scale, c.voxel_space[1] * scale, c.voxel_space[2] * scale);
                if constexpr (G == 1) {
                    for (float z = -kr; z <= kr; z += 1.0f)
                        for (float y = -kr; y <= kr; y += 1.0f)
                            for (float x = -kr; x <= kr; x += 1.0f) {
                                const Vec3 q = v3(surf.x + x * sc.x, surf.y + y * sc.y, surf.z + z * sc.z);
                                dsum += fminf(density_at<DF, shade_source(SRC)>(c, dens, q), c.ao_max);
                            }
                } else { // the cube's taps in loop order, G at a time; each offset by the loop's own additions
                    int m = 0;
                    for (float x = -kr; x <= kr; x += 1.0f) ++m;
                    const int n = m * m * m, rank = (int)(threadIdx.x & (G - 1));
                    for (int base = 0; base < n; base += G) {
                        const int i = base + rank;
                        float d = 0.0f;
                        if (i < n) {
                            const float x = group_t(-kr, 1.0f, i % m), y = group_t(-kr, 1.0f, (i / m) % m),
                                        z = group_t(-kr, 1.0f, i / (m * m));
                            const Vec3 q = v3(surf.x + x * sc.x, surf.y + y * sc.y, surf.z + z * sc.z);
                            d = density_at<DF, shade_source(SRC)>(c, dens, q);
                        }
                        int cs[G];
                        float vs[G];
                        group_outcomes<G>(0, d, cs, vs);
#pragma unroll
                        for (int j = 0; j < G; ++j)
                            if (base + j < n) dsum += fminf(vs[j], c.ao_max);
                    }
                }
                taps = c.ao_kernel * c.ao_kernel * c.ao_kernel;
            }
            if (TAPE) tape->dsum = dsum;
            occlusion *= powf(1.0f - dsum / taps, c.ao_exp);
        }
        // packUnorm4x8 clamp (ppll.glsl:32); NaN -> 0
        out = make_float4(__saturatef(shading.x * occlusion), __saturatef(shading.y * occlusion),
                          __saturatef(shading.z * occlusion), __saturatef(coverage));
        out_depth = clip_depth(c, surf);
    }
}

// The fragment of pixel (px, py) of the c.W x c.H view: colour + coverage
// and depth.  depth_at points at the pixel's depth-buffer value (NULL: 1.0).
// TAPE = true also records the pixel's PixelTape and the march's t every K
// iterations into ckpt[0, nckpt) (the checkpoints the adjoint replays from).
// G > 1: the ray group's form (G lanes, the same pixel in each).
template <int DF, int TF, bool TAPE = false, int SRC = kSampleMemory, int G = 1>
__device__ __forceinline__ void march_pixel(const RayConsts& c, const typename DensityTexel<DF>::T* __restrict__ dens,
                                            const void* __restrict__ tang, const uint32_t* __restrict__ occ,
                                            const float* depth_at, int px, int py, float4& out, float& out_depth,
                                            PixelTape* tape = nullptr, float* ckpt = nullptr, uint32_t K = 1,
                                            uint32_t nckpt = 0)
{
    out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    out_depth = 1.0f;
    if (TAPE) {
        tape->surf[0] = tape->surf[1] = tape->surf[2] = 0.0f;
        tape->acc = 0.0f;
        tape->occl_s = 1.0f;
        tape->dsum = 0.0f;
        tape->n = 0;
        tape->flags = 0;
    }
    Vec3 start, end;
    if (ray_entry(c, px, py, start, end)) {
        const float db = depth_at ? *depth_at : 1.0f;
        const bool depth_test = !(clip_depth(c, end) < db);

        // ---- volume_surface (volume_rendering.glsl:19-52) --------------------
        const float step = 1.0f / c.steps;
        const bool jump = c.steps_pow2 && !depth_test;
        float us[3], ue[3], du[3];
        texel_coords(c, start, us);
        texel_coords(c, end, ue);
        du[0] = ue[0] - us[0];
        du[1] = ue[1] - us[1];
        du[2] = ue[2] - us[2];
        float inv_du[3];
        reciprocals(du, inv_du);
        float acc = 0.0f;
        Vec3 surf = v3(0.0f, 0.0f, 0.0f), entry = v3(0.0f, 0.0f, 0.0f);
        bool found = false, entered = false;
        uint32_t k = 0; // iterations (TAPE only)
        static_assert(G == 1 || !TAPE, "the adjoint's tape records one lane's march");
        if constexpr (G > 1) { // G samples at a time, replayed in order
            const int rank = (int)(threadIdx.x & (G - 1));
            float t_surf = 0.0f, t_entry = 0.0f;
            bool at_surf = false;
            for (float t = 0.0f; t < 1.0f;) {
                const float tr = group_t(t, step, rank);
                int code = 4;
                float val = 0.0f;
                if (tr < 1.0f) {
                    const Vec3 P = mix(start, end, tr);
                    if (depth_test && db < clip_depth(c, P)) {
                        code = 3;
                    } else {
                        float u[3], lo[3], hi[3];
                        texel_coords(c, P, u);
                        code = classify(c, occ, u, inv_du, lo, hi);
                        if (code == 1) val = jump ? steps_inside(u, inv_du, lo, hi, c.steps) : 0.0f;
                        else if (code == 0) val = density_at<DF, march_source(SRC)>(c, dens, P);
                    }
                }
                int cs[G];
                float vs[G];
                group_outcomes<G>(code, val, cs, vs);
                bool stop = false, jumped = false;
                float tc = t;
#pragma unroll
                for (int j = 0; j < G; ++j) {
                    if (stop || jumped) continue;
                    if (cs[j] >= 2) {
                        stop = true;
                    } else if (cs[j] == 1) {
                        if (vs[j] >= 1.0f) {
                            t = fmaf(vs[j], step, tc);
                            jumped = true;
                        } else {
                            tc += step;
                        }
                    } else {
                        const float rho = vs[j];
                        acc += rho;
                        if (rho != 0.0f) {
                            if (acc <= c.iso) {
                                t_surf = tc;
                                at_surf = true;
                            }
                            if (acc >= c.iso) found = true;
                            if (!entered) {
                                t_entry = tc;
                                entered = true;
                            }
                            if (acc > c.iso && c.lod * (acc / c.iso) * c.alpha >= 1.0f) stop = true; // outputs final
                        }
                        if (!stop) tc += step;
                    }
                }
                if (stop) break;
                if (!jumped) t = tc;
            }
            // the points the serial loop kept, from their t (mix gives the same point for the same t)
            if (at_surf) surf = mix(start, end, t_surf);
            if (entered) entry = mix(start, end, t_entry);
        } else
        for (float t = 0.0f; t < 1.0f;) {
            if (TAPE && !jump && k % K == 0 && k / K < nckpt) ckpt[k / K] = t;
            const Vec3 P = mix(start, end, t);
            if (depth_test && db < clip_depth(c, P)) break;
            float u[3], lo[3], hi[3];
            texel_coords(c, P, u);
            const int z = classify(c, occ, u, inv_du, lo, hi);
            if (z == 2) break; // left the grid: every later sample adds exactly 0
            if (z == 1) {      // exactly 0: acc and the decisions are unchanged
                const float n = jump ? steps_inside(u, inv_du, lo, hi, c.steps) : 0.0f;
                t = n >= 1.0f ? fmaf(n, step, t) : t + step;
                if (TAPE) k += n >= 1.0f ? (uint32_t)n : 1u;
                continue;
            }
            const float rho = density_at<DF, march_source(SRC)>(c, dens, P);
            acc += rho;
            if (rho != 0.0f) {
                if (acc <= c.iso) surf = P;
                if (acc >= c.iso) found = true;
                if (!entered) { entry = P; entered = true; }
                if (acc > c.iso && c.lod * (acc / c.iso) * c.alpha >= 1.0f) { // outputs final
                    if (TAPE) ++k;
                    break;
                }
            }
            t += step;
            if (TAPE) ++k;
        }
        if (!found && entered) surf = entry;
        if (TAPE) {
            if (jump) // power-of-two steps: t = i * step exactly
                for (uint32_t m = 0; m * K < k && m < nckpt; ++m) ckpt[m] = (float)(m * K) * step;
            tape->surf[0] = surf.x;
            tape->surf[1] = surf.y;
            tape->surf[2] = surf.z;
            tape->acc = acc;
            tape->n = k;
            tape->flags = kTapeHit;
        }
        shade_fragment<DF, TF, TAPE, SRC, G>(c, dens, tang, occ, surf, acc, out, out_depth, tape);
    }
}

inline bool invert4(const double m[16], double inv[16])
{
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) {
            a[r][k] = m[k * 4 + r];
            a[r][k + 4] = r == k ? 1.0 : 0.0;
        }
    for (int k = 0; k < 4; ++k) {
        int piv = k;
        for (int r = k + 1; r < 4; ++r)
            if (std::fabs(a[r][k]) > std::fabs(a[piv][k])) piv = r;
        if (a[piv][k] == 0.0) return false;
        if (piv != k)
            for (int j = 0; j < 8; ++j) std::swap(a[k][j], a[piv][j]);
        const double d = a[k][k];
        for (int j = 0; j < 8; ++j) a[k][j] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != k) {
                const double f = a[r][k];
                for (int j = 0; j < 8; ++j) a[r][j] -= f * a[k][j];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) inv[k * 4 + r] = a[r][k + 4];
    return true;
}

inline vkhr_status make_consts(vkhr_ctx* ctx, const vkhr_raymarch_params* p, RayConsts& c)
{
    if (p->width <= 0 || p->height <= 0) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "width/height must be > 0");
    if (!(p->raycast_steps > 0.0f) || !(p->raycast_steps <= kMaxSteps))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "raycast_steps must be in (0, 2^20]");
    const float sst = p->shadow_steps > 0.0f ? p->shadow_steps : p->raycast_steps;
    if (!(sst <= kMaxSteps)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "shadow_steps must be <= 2^20");
    if (p->ao_directions < 0 || p->ao_directions > kMaxAoDirections)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "ao_directions must be in [0, 32]");
    if (p->ao_directions == 0 && !(p->ao_kernel_size >= 2.0f && p->ao_kernel_size <= 16.0f))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "ao_kernel_size must be in [2, 16]");
    if (!std::isfinite(p->spec_exponent2) || !std::isfinite(p->spec_shift[0]) || !std::isfinite(p->spec_shift[1]))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "spec_exponent2 and spec_shift must be finite");
    if (!(p->isosurface > 0.0f)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "isosurface must be > 0");
    if (p->density_format < 0 || p->density_format > 2 || p->tangent_format < 0 || p->tangent_format > 1)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown texel format");
    for (int k = 0; k < 3; ++k) {
        if (p->volume_resolution[k] <= 0) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "volume_resolution must be > 0");
        if (!(p->volume_bounds.size[k] > 0.0f) || !std::isfinite(p->volume_bounds.size[k]))
            return vkhr_fail(ctx, VKHR_ERR_DEGENERATE_AABB, "every AABB extent must be finite and > 0");
    }
    c.W = p->width;
    c.H = p->height;
    double pv[16], inv[16];
    for (int col = 0; col < 4; ++col)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += (double)p->projection[k * 4 + r] * (double)p->view[col * 4 + k];
            pv[col * 4 + r] = s;
        }
    if (!invert4(pv, inv)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "projection * view is singular");
    for (int i = 0; i < 16; ++i) c.pv[i] = (float)pv[i];
    // rays: inverse(P V) (nx, ny, 1, 1) = (num, w), affine in (nx, ny), with
    // nx = 2 (px + 0.5) / W - 1 (likewise ny); the direction num - camera * w
    // (inv is column-major: inv[col * 4 + row]), in the pixel basis, each
    // coefficient split into float hi + lo
    {
        const double sx = 2.0 / (double)p->width, ox = 1.0 / (double)p->width - 1.0;
        const double sy = 2.0 / (double)p->height, oy = 1.0 / (double)p->height - 1.0;
        auto split = [](double v, float out[2]) {
            out[0] = (float)v;
            out[1] = (float)(v - (double)out[0]);
        };
        for (int k = 0; k < 3; ++k) {
            const double cam = (double)p->camera_position[k];
            const double an = inv[0 * 4 + k] - cam * inv[0 * 4 + 3];                            // d/dnx
            const double am = inv[1 * 4 + k] - cam * inv[1 * 4 + 3];                            // d/dny
            const double a0 = inv[2 * 4 + k] + inv[3 * 4 + k] - cam * (inv[2 * 4 + 3] + inv[3 * 4 + 3]);
            split(a0 + an * ox + am * oy, c.ray_dir[k][0]);
            split(an * sx, c.ray_dir[k][1]);
            split(am * sy, c.ray_dir[k][2]);
        }
        const double wn = inv[0 * 4 + 3], wm = inv[1 * 4 + 3], w0 = inv[2 * 4 + 3] + inv[3 * 4 + 3];
        c.ray_w[0] = (float)(w0 + wn * ox + wm * oy);
        c.ray_w[1] = (float)(wn * sx);
        c.ray_w[2] = (float)(wm * sy);
    }
    for (int k = 0; k < 3; ++k) {
        c.cam[k] = p->camera_position[k];
        c.lo[k] = p->volume_bounds.origin[k];
        c.hi[k] = p->volume_bounds.origin[k] + p->volume_bounds.size[k];
        c.res[k] = p->volume_resolution[k];
        const double s = (double)p->volume_resolution[k] / (double)p->volume_bounds.size[k];
        c.tsc[k] = (float)s;
        c.tbias[k] = (float)(-(double)p->volume_bounds.origin[k] * s - 0.5);
        c.voxel_space[k] = p->volume_bounds.size[k] / (float)p->volume_resolution[k];
        c.light[k] = p->light_origin[k];
        c.intensity[k] = p->light_intensity[k];
        c.color[k] = p->hair_color[k];
    }
    c.radius = p->volume_bounds.radius;
    c.alpha = p->hair_alpha;
    c.exponent = p->hair_exponent;
    c.iso = p->isosurface;
    c.kd = p->kd;
    c.steps = p->raycast_steps;
    c.shadow_steps = sst;
    c.thickness = p->shadow_thickness;
    c.ao_kernel = p->ao_kernel_size;
    c.ao_radius = p->occlusion_radius;
    c.ao_exp = p->ao_exponent;
    c.ao_max = p->ao_max;
    // lod() of scheme.glsl:7-11 for the camera's look-at distance
    if (p->renderer == VKHR_RENDERER_RASTERIZER) c.lod = 0.0f;
    else if (p->renderer == VKHR_RENDERER_RAYMARCHER) c.lod = 1.0f;
    else {
        float t = (p->look_at_distance - p->magnified_distance) / (p->minified_distance - p->magnified_distance);
        t = std::min(std::max(t, 0.0f), 1.0f);
        c.lod = t * t * (3.0f - 2.0f * t);
    }
    c.shading_model = p->shading_model;
    c.deep_shadows_on = p->deep_shadows_on;
    auto pow2 = [](float x) {
        int e;
        return std::frexp(x, &e) == 0.5f;
    };
    c.steps_pow2 = pow2(c.steps) ? 1 : 0;
    c.shadow_pow2 = pow2(c.shadow_steps) ? 1 : 0;
    for (int k = 0; k < 3; ++k) c.nb[k] = (c.res[k] + kBrick) / kBrick;
    c.tex = 0;
    c.gshift = 0;
    c.exponent2 = p->spec_exponent2 > 0.0f ? p->spec_exponent2 : 0.0f;
    c.shift[0] = p->spec_shift[0];
    c.shift[1] = p->spec_shift[1];
    // directional AO: Fibonacci-sphere directions (y polar) at the reach of
    // the reference's 8-tap cube, radius * sqrt(3) voxels, in world units
    c.ao_n = p->ao_directions;
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < kMaxAoDirections; ++i)
        for (int k = 0; k < 3; ++k) c.ao_off[i][k] = 0.0f;
    for (int i = 0; i < c.ao_n; ++i) {
        const double y = 1.0 - (2.0 * i + 1.0) / (double)c.ao_n, r = std::sqrt(1.0 - y * y);
        const double phi = (double)i * pi * (3.0 - std::sqrt(5.0));
        const double d[3] = {r * std::cos(phi), y, r * std::sin(phi)};
        const double reach = (double)p->occlusion_radius * std::sqrt(3.0);
        for (int k = 0; k < 3; ++k)
            c.ao_off[i][k] = (float)(d[k] * reach * (double)p->volume_bounds.size[k] / (double)p->volume_resolution[k]);
    }
    return VKHR_OK;
}

} // namespace
