// glmshim/glm/glm.hpp -- TEST INFRASTRUCTURE ONLY.
//
// A minimal stand-in for the glm API subset that vkhr's voxelizer source
// (src/vkhr/scene_graph/hair_style.cc and include/vkhr/scene_graph/hair_style.hh)
// uses, written for this project so that the reference's own voxelizer can be
// compiled unmodified into oracle/_ref and used to pin the C oracle.  glm is an
// empty git submodule in the reference checkout.
//
// Semantics are glm's documented component-wise ones, in IEEE FP32:
//   min(x, y) = y < x ? y : x        max(x, y) = x < y ? y : x
//   floor/abs per component           compMax(v) = max(max(v.x, v.y), v.z)
//   dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z
//   length(v) = sqrt(dot(v, v))       normalize(v) = v * (1 / sqrt(dot(v, v)))
//   integer vectors from float vectors convert each component with static_cast.
#ifndef VKHR_GLMSHIM_GLM_HPP
#define VKHR_GLMSHIM_GLM_HPP

#include <cmath>
#include <cstdint>
#include <cstddef>
#include <limits>

namespace glm {

inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }

struct vec3 {
    float x, y, z;
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    template <class X, class Y, class Z>
    vec3(X a, Y b, Z c) : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

struct vec4 {
    float x, y, z, w;
    vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    vec4(const vec3& v, float s) : x(v.x), y(v.y), z(v.z), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

template <class T>
struct tvec3i {
    T x, y, z;
    tvec3i() : x(0), y(0), z(0) {}
    tvec3i(const vec3& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
};
typedef tvec3i<std::int8_t> i8vec3;
typedef tvec3i<int> ivec3;

struct i8vec4 {
    std::int8_t x, y, z, w;
    i8vec4() : x(0), y(0), z(0), w(0) {}
    i8vec4(int a, int b, int c, int d)
        : x(static_cast<std::int8_t>(a)), y(static_cast<std::int8_t>(b)),
          z(static_cast<std::int8_t>(c)), w(static_cast<std::int8_t>(d)) {}
};

inline vec3 floor(const vec3& v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v * (1.0f / std::sqrt(dot(v, v))); }

} // namespace glm

#endif
