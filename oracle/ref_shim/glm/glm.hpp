// oracle/ref_shim/glm/glm.hpp — TEST INFRASTRUCTURE ONLY.
//
// A minimal, project-written stand-in for the header-only glm library, which the
// reference pins through vcpkg (native/vcpkg.json:6-15) and which is not installed
// here. It provides just the types and functions that the reference's
// native/src/engine/sdf/cuda_types.hpp and native/src/core/math_utils.cuh use on
// the host: vec3 / vec4 / ivec3, + - * (scalar), dot, cross, min, max.
// Arithmetic follows glm's component order: dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
// cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y).
// Constructors are defaulted so the types stay trivially constructible.
#pragma once
#include <algorithm>

namespace glm {

struct vec3 {
    float x, y, z;
    vec3() = default;
    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 min(const vec3& a, const vec3& b) {
    return vec3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z));
}
inline vec3 max(const vec3& a, const vec3& b) {
    return vec3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z));
}

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

struct ivec3 {
    int x, y, z;
    ivec3() = default;
    constexpr explicit ivec3(int s) : x(s), y(s), z(s) {}
    constexpr ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }

}  // namespace glm
