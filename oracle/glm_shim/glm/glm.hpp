// Minimal, project-written stand-in for the subset of GLM that the reference SPH core
// uses (glm::vec3 / glm::ivec3 / glm::vec2, component-wise arithmetic, dot, length).
//
// TEST INFRASTRUCTURE ONLY: this header exists so that the reference sources
// (src/particle.cpp, src/kernels.cpp, src/spatial_hash.cpp, src/sph_engine.cpp) can be
// compiled unmodified into the oracle library oracle/_ref/libsph_ref.so.  GLM itself is
// not vendored by the reference (README.md:267-268) and is not installed here.
//
// Semantics follow GLM's documented behaviour for the operations the reference calls:
//   * every vector operator is component-wise, evaluated in float;
//   * scalar * vec and vec * scalar multiply each component, vec / scalar DIVIDES each
//     component (no reciprocal multiply);
//   * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z, with each product rounded first;
//   * length(v) = sqrt(dot(v, v)).
// The default constructor zero-initialises (what std::vector<vec3>::resize produces
// with GLM's defaulted constructor under value-initialisation).
#pragma once
#include <cmath>
#include <cstdint>

namespace glm {

struct vec2 {
    float x, y;
    vec2() : x(0.0f), y(0.0f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    float x, y, z;
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& v, float s) { return vec3(v.x * s, v.y * s, v.z * s); }
inline vec3 operator*(float s, const vec3& v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 operator/(const vec3& v, float s) { return vec3(v.x / s, v.y / s, v.z / s); }
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }

inline float dot(const vec3& a, const vec3& b) {
    const vec3 t = a * b;
    return (t.x + t.y) + t.z;
}
inline float dot(const vec2& a, const vec2& b) {
    const float tx = a.x * b.x;
    const float ty = a.y * b.y;
    return tx + ty;
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }

}  // namespace glm
