// glslshim/glsl.hpp -- TEST INFRASTRUCTURE ONLY.
//
// Just enough of GLSL 4.60 (types, built-ins, a software sampler3D, storage
// images) for the reference's raymarch shader (share/shaders/volumes/
// volume.frag and its includes) and its PPLL resolve (share/shaders/
// transparency/resolve.comp, ppll.glsl) to compile as C++17 and run on the
// CPU in strict FP32.  Written
// for this project; everything lives in namespace glsl so that unqualified
// calls inside the shader code resolve to these overloads only.
//
// sampler3D follows the Vulkan sampling rules the reference configures
// (VK_FILTER_LINEAR, CLAMP_TO_BORDER, src/vkhr/rasterizer/hair_style.cc:79-85):
// u = s*size - 0.5, i0 = floor(u), alpha = frac(u), border texels read 0.
// R8_UNORM texels read c/255, R8G8B8A8_SNORM texels read max(c/127, -1).
// The weights are FP32 here (a GPU's texture unit uses 8-bit fractions).
#ifndef VKHR_GLSLSHIM_HPP
#define VKHR_GLSLSHIM_HPP

#include <cmath>
#include <cstdint>
#include <cstddef>

namespace glsl {

typedef unsigned int uint;

struct vec2 {
    float x, y;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct ivec2;
struct ivec3;
struct uvec2;

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        vec2 st;
        vec2 xy;
    };
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const ivec3& v);
    vec3 operator-() const { return vec3(-x, -y, -z); }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        vec3 xyz;
        vec2 xy;
    };
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float p, float q, float s, float t) : x(p), y(q), z(s), w(t) {}
    vec4(const vec3& v, float t) : x(v.x), y(v.y), z(v.z), w(t) {}
};

struct ivec2 {
    int x, y;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
    explicit ivec2(const uvec2& v);
    operator vec2() const { return vec2((float)x, (float)y); }
};

struct ivec3 {
    int x, y, z;
    ivec3() = default;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};

inline vec3::vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}

struct mat4 {
    vec4 c[4]; // columns, as glm::mat4 stores them
};

// ---- arithmetic ------------------------------------------------------------
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator/(vec2 a, float s) { return vec2(a.x / s, a.y / s); }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline vec4& operator+=(vec4& a, vec4 b) { a = a + b; return a; }

// GLSL matrix products: component k of M*v is sum_j M[j][k] * v[j].
inline vec4 operator*(const mat4& m, vec4 v)
{
    vec4 r;
    r.x = m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w;
    r.y = m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w;
    r.z = m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w;
    r.w = m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w;
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b)
{
    mat4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = a * b.c[j];
    return r;
}

// ---- built-ins -------------------------------------------------------------
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float clamp(float x, float a, float b) { return min(max(x, a), b); }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline float smoothstep(float e0, float e1, float x)
{
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ---- textures --------------------------------------------------------------
enum { TEX_R8_UNORM = 0, TEX_R32_UINT_AS_FLOAT = 1, TEX_R32F = 2, TEX_RGBA8_SNORM = 10, TEX_RGBA32F = 11 };

struct sampler3D {
    const void* data;
    int format;
    int n[3];
};

inline vec4 texel3D(const sampler3D& s, long i, long j, long k)
{
    if (i < 0 || j < 0 || k < 0 || i >= s.n[0] || j >= s.n[1] || k >= s.n[2]) return vec4(0.0f, 0.0f, 0.0f, 1.0f);
    std::size_t at = (std::size_t)i + (std::size_t)s.n[0] * ((std::size_t)j + (std::size_t)s.n[1] * (std::size_t)k);
    switch (s.format) {
    case TEX_R8_UNORM: return vec4((float)((const std::uint8_t*)s.data)[at] / 255.0f, 0.0f, 0.0f, 1.0f);
    case TEX_R32_UINT_AS_FLOAT: return vec4((float)((const std::uint32_t*)s.data)[at], 0.0f, 0.0f, 1.0f);
    case TEX_R32F: return vec4(((const float*)s.data)[at], 0.0f, 0.0f, 1.0f);
    case TEX_RGBA8_SNORM: {
        const std::int8_t* q = (const std::int8_t*)s.data + 4 * at;
        float c[4];
        for (int a = 0; a < 4; ++a) c[a] = max((float)q[a] / 127.0f, -1.0f);
        return vec4(c[0], c[1], c[2], c[3]);
    }
    default: {
        const float* f = (const float*)s.data + 4 * at;
        return vec4(f[0], f[1], f[2], f[3]);
    }
    }
}

inline vec4 texture(const sampler3D& s, vec3 uvw)
{
    float st[3] = {uvw.x, uvw.y, uvw.z};
    long i0[3];
    float al[3];
    for (int c = 0; c < 3; ++c) {
        float u = st[c] * (float)s.n[c] - 0.5f;
        if (!(u > -2.0f && u < (float)(s.n[c] + 1))) return vec4(0.0f, 0.0f, 0.0f, 1.0f);
        float f = std::floor(u);
        i0[c] = (long)f;
        al[c] = u - f;
    }
    vec4 acc(0.0f);
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                float w = (dx ? al[0] : 1.0f - al[0]) * (dy ? al[1] : 1.0f - al[1]) * (dz ? al[2] : 1.0f - al[2]);
                acc += texel3D(s, i0[0] + dx, i0[1] + dy, i0[2] + dz) * w;
            }
    return acc;
}

inline ivec3 textureSize(const sampler3D& s, int) { return ivec3(s.n[0], s.n[1], s.n[2]); }

// 2D samplers appear only in the shadow-map code paths that volume.frag
// compiles but never calls.
struct sampler2D { int n[2]; };
inline vec4 texture(const sampler2D&, vec2) { return vec4(1.0f); }
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.n[0], s.n[1]); }

struct subpassInput { int unused; };

// ---- compute shaders and storage images --------------------------------------
// Enough for share/shaders/transparency/resolve.comp and ppll.glsl.  An
// rgba8 image holds one 32-bit word per texel, red in the low byte; its
// loads and stores convert as unpackUnorm4x8 / packUnorm4x8 do (Vulkan's
// UNORM conversions: c / 255, and clamp to [0, 1] then the nearest of the
// two closest codes -- ties, which the specs leave open, go to even here).
struct uvec2 {
    uint x, y;
};
struct uvec3 {
    union {
        struct { uint x, y, z; };
        uvec2 xy;
    };
    uvec3() = default;
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
struct uvec4 {
    union {
        struct { uint x, y, z, w; };
        struct { uint r, g, b, a; };
    };
    uvec4() = default;
    uvec4(uint p, uint q, uint s, uint t) : x(p), y(q), z(s), w(t) {}
};
inline ivec2::ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}

inline vec4 mix(vec4 x, vec4 y, float a) { return x * (1.0f - a) + y * a; }

inline vec4 unpackUnorm4x8(uint c)
{
    return vec4((float)(c & 0xffu) / 255.0f, (float)((c >> 8) & 0xffu) / 255.0f, (float)((c >> 16) & 0xffu) / 255.0f,
                (float)((c >> 24) & 0xffu) / 255.0f);
}

inline uint unorm8_code(float x)
{
    x = x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f;
    return (uint)std::nearbyint(x * 255.0f);
}

inline uint packUnorm4x8(vec4 v)
{
    return unorm8_code(v.x) | unorm8_code(v.y) << 8 | unorm8_code(v.z) << 16 | unorm8_code(v.w) << 24;
}

struct uimage2D { // r32ui
    uint* data;
    int width, height;
};
struct image2D { // rgba8
    uint* data;
    int width, height;
};

inline std::size_t texel_at(int width, ivec2 p) { return (std::size_t)p.y * (std::size_t)width + (std::size_t)p.x; }
inline uvec4 imageLoad(const uimage2D& im, ivec2 p) { return uvec4(im.data[texel_at(im.width, p)], 0u, 0u, 1u); }
inline uint imageAtomicExchange(uimage2D& im, ivec2 p, uint v)
{
    uint& t = im.data[texel_at(im.width, p)];
    const uint old = t;
    t = v;
    return old;
}
inline vec4 imageLoad(const image2D& im, ivec2 p) { return unpackUnorm4x8(im.data[texel_at(im.width, p)]); }
inline void imageStore(image2D& im, ivec2 p, vec4 v) { im.data[texel_at(im.width, p)] = packUnorm4x8(v); }

inline uint atomicAdd(uint& mem, uint v)
{
    const uint old = mem;
    mem += v;
    return old;
}

} // namespace glsl

#endif
