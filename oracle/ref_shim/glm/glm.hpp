// oracle/ref_shim/glm/glm.hpp — TEST INFRASTRUCTURE ONLY.
//
// A minimal, project-written stand-in for the header-only glm library, which the
// reference pins through vcpkg (native/vcpkg.json:6-15) and which is not installed
// here. It provides just the types and functions that the reference's
// native/src/engine/sdf/cuda_types.hpp, native/src/core/math_utils.cuh and
// native/src/engine/sdf/cuda_rasterizer.{hpp,cu} use: vec3 / vec4 / ivec3 / mat4,
// + - * / (scalar), dot, cross, min, max. Under nvcc every function is
// __host__ __device__, as glm's own functions are when compiled by nvcc.
// Arithmetic follows glm's component order: dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
// cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
// min(a, b) = b < a ? b : a, max(a, b) = a < b ? b : a per component.
// Constructors are defaulted so the types stay trivially constructible (the reference
// declares __shared__ arrays of CudaTriangle).
#pragma once

#if defined(__CUDACC__)
#define GLMS_HD __host__ __device__ __forceinline__
#else
#define GLMS_HD inline
#endif

namespace glm {

struct vec3 {
    float x, y, z;
    vec3() = default;
    GLMS_HD constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    GLMS_HD constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    GLMS_HD vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    GLMS_HD vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    GLMS_HD vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    GLMS_HD vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};
GLMS_HD vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
GLMS_HD vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
GLMS_HD vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
GLMS_HD vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
GLMS_HD vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
GLMS_HD vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
GLMS_HD vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
GLMS_HD float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GLMS_HD vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
GLMS_HD float min(float a, float b) { return b < a ? b : a; }
GLMS_HD float max(float a, float b) { return a < b ? b : a; }
GLMS_HD int min(int a, int b) { return b < a ? b : a; }
GLMS_HD int max(int a, int b) { return a < b ? b : a; }
GLMS_HD vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
GLMS_HD vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    GLMS_HD constexpr explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    GLMS_HD constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

// Only named in declarations of the reference's camera / viewport entry points.
struct mat4 {
    vec4 c[4];
};

struct ivec3 {
    int x, y, z;
    ivec3() = default;
    GLMS_HD constexpr explicit ivec3(int s) : x(s), y(s), z(s) {}
    GLMS_HD constexpr ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};
GLMS_HD ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
GLMS_HD ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }

}  // namespace glm
