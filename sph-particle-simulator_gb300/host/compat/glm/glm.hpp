// GLM-compatible vector types for building the drop-in engine where GLM itself is not
// installed.  The build adds this directory with -idirafter, so an installed GLM (which
// the reference's users have) always takes precedence.  Provides the subset the engine's
// public API uses: glm::vec3 / glm::vec2 / glm::ivec3, component-wise arithmetic,
// dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z and length(v) = sqrt(dot(v, v)).
#pragma once
#include <cmath>

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

inline vec3 operator+(const vec3& a, const vec3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(const vec3& a, const vec3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(const vec3& a, const vec3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator-(const vec3& a) { return {-a.x, -a.y, -a.z}; }
inline vec3 operator*(const vec3& v, float s) { return {v.x * s, v.y * s, v.z * s}; }
inline vec3 operator*(float s, const vec3& v) { return {s * v.x, s * v.y, s * v.z}; }
inline vec3 operator/(const vec3& v, float s) { return {v.x / s, v.y / s, v.z / s}; }
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }

inline float dot(const vec3& a, const vec3& b) {
    const float px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    return (px + py) + pz;
}
inline float dot(const vec2& a, const vec2& b) {
    const float px = a.x * b.x, py = a.y * b.y;
    return px + py;
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }

}  // namespace glm
