// oracle/ref_math_wrap.cpp — TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's OWN host/device geometry primitives, exactly as they lie
// in the reference tree (native/src/core/math_utils.cuh:43-132, included from there
// by oracle/build_ref.sh), against the project-written glm stand-in in
// oracle/ref_shim/. The result, oracle/_ref/libref_math.so, is a checker: it pins the
// oracle's restated primitives bit for bit (tests/golden/make_golden.py). It exists
// only where the reference tree is present and never ships with the product.
#include "core/math_utils.cuh"

extern "C" {

float ref_point_triangle_distance_sq(const float* p, const float* a, const float* b, const float* c) {
    glm::vec3 cl;
    return rhizome::point_triangle_distance_sq(glm::vec3(p[0], p[1], p[2]), glm::vec3(a[0], a[1], a[2]),
                                               glm::vec3(b[0], b[1], b[2]), glm::vec3(c[0], c[1], c[2]), cl);
}

float ref_triangle_solid_angle(const float* p, const float* a, const float* b, const float* c) {
    return rhizome::triangle_solid_angle(glm::vec3(p[0], p[1], p[2]), glm::vec3(a[0], a[1], a[2]),
                                         glm::vec3(b[0], b[1], b[2]), glm::vec3(c[0], c[1], c[2]));
}

void ref_ptd_batch(const float* pts, const float* tris9, long long n, float* out) {
    for (long long i = 0; i < n; ++i)
        out[i] = ref_point_triangle_distance_sq(pts + 3 * i, tris9 + 9 * i, tris9 + 9 * i + 3, tris9 + 9 * i + 6);
}

void ref_solid_angle_batch(const float* pts, const float* tris9, long long n, float* out) {
    for (long long i = 0; i < n; ++i)
        out[i] = ref_triangle_solid_angle(pts + 3 * i, tris9 + 9 * i, tris9 + 9 * i + 3, tris9 + 9 * i + 6);
}

}  // extern "C"
