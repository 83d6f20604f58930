// gbsdf_device.cuh — device-side geometry and eikonal arithmetic for the GB300
// mesh-to-SDF engine.
//
// Every translation unit of the engine is compiled with -fmad=false: products
// and sums round separately, in the operation order of the reference's
// expressions (native/src/core/math_utils.cuh, native/src/engine/sdf/
// cuda_rasterizer.cu), and every fused multiply-add is written out with
// __fmaf_rn. The parity edge functions and hit heights and the Godunov update
// fuse exactly the products that the reference's own build (nvcc's default
// contraction) fuses, so they are bit-identical to the reference's kernels; the
// band distances round as a contraction-free evaluation (within 1e-5 voxel of
// the reference's). Where speed matters more than bit-identity (the FP32 winding
// sum, whose sign decisions are re-checked in FP64 near the threshold), fused
// multiply-adds are chosen freely.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbsdf {

// ---- constants of the reference path (cuda_rasterizer.cu:74-82, :298-299, :825, :1010, :1027)
constexpr int kBandVoxels = 8;
constexpr int kParityMaxHits = 128;
constexpr float kFarSentinel = 1e30f;
constexpr int kVerifySamples = 4096;
constexpr int kProbeGens = 3;
constexpr int kMaxSitesPerProbe = 64;
constexpr int kPatchRadius = 24;
constexpr int kSup = 4;
constexpr int kMaxRounds = 8;
constexpr int kMaxExtraRounds = 16;
constexpr float kJX = 0.037f;
constexpr float kJY = 0.051f;
constexpr float kInv4Pi = 0.07957747154594767f;
constexpr float kRecheckBand = 0.05f;  // FP64 re-evaluation when | |w| - 0.5 | < this
// A voxel within this many voxels of the surface lies on it: its winding number is 0.5 in
// exact arithmetic (inside by |w| >= 0.5), while any floating-point sum of it is noise.
constexpr float kSurfaceTolVoxels = 1e-5f;
// The exact-signs modes cast near-lattice rays (offset 3.7e-4 h, 5.1e-4 h) and treat
// voxels within 1e-3 voxel of the surface as on it.
constexpr float kSurfaceTolExactSigns = 1e-3f;
// A triangle term's sign is uncertain when |det| < this * |a||b||c| and the point
// projects inside the triangle (denominator < 0): such voxels are decided in FP64.
constexpr float kCoplanarRel = 1e-4f;
constexpr unsigned long long kFastMinVoxels = 32ull * 1024ull * 1024ull;

// Brick edge of the band splat and lattice strip width of the parity pass.
constexpr int kBrick = 8;
constexpr int kStrip = 32;

struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__host__ __device__ __forceinline__ f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 mul(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
// glm::dot on vec3: (x*x' + y*y') + z*z'
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Exact point-triangle squared distance, point_triangle_distance_sq
// (math_utils.cuh:43-106): Ericson's seven Voronoi regions, same branch order.
__device__ __forceinline__ float ptd_sq(f3 p, f3 a, f3 b, f3 c) {
    f3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return dot(ap, ap);
    f3 bp = sub(p, b);
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return dot(bp, bp);
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        f3 df = sub(p, add(a, mul(ab, v)));
        return dot(df, df);
    }
    f3 cp = sub(p, c);
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return dot(cp, cp);
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        f3 df = sub(p, add(a, mul(ac, w)));
        return dot(df, df);
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        f3 df = sub(p, add(b, mul(sub(c, b), w)));
        return dot(df, df);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    f3 df = sub(p, add(add(a, mul(ab, v)), mul(ac, w)));
    return dot(df, df);
}

// Triangle solid angle (Van Oosterom-Strackee), triangle_solid_angle
// (math_utils.cuh:109-132), FP32 with explicit FMAs: the winding sum's sign is
// decided exactly by re-evaluating in FP64 near the threshold, so this form is
// free to be fast.
__device__ __forceinline__ float solid_angle_fast(f3 p, f3 v0, f3 v1, f3 v2, bool& amb) {
    float ax = v0.x - p.x, ay = v0.y - p.y, az = v0.z - p.z;
    float bx = v1.x - p.x, by = v1.y - p.y, bz = v1.z - p.z;
    float cx = v2.x - p.x, cy = v2.y - p.y, cz = v2.z - p.z;
    float la = sqrtf(__fmaf_rn(az, az, __fmaf_rn(ay, ay, ax * ax)));
    float lb = sqrtf(__fmaf_rn(bz, bz, __fmaf_rn(by, by, bx * bx)));
    float lc = sqrtf(__fmaf_rn(cz, cz, __fmaf_rn(cy, cy, cx * cx)));
    if (la <= 1e-6f || lb <= 1e-6f || lc <= 1e-6f) return 0.0f;
    float det = __fmaf_rn(az, __fmaf_rn(bx, cy, -(by * cx)),
                          __fmaf_rn(-ay, __fmaf_rn(bx, cz, -(bz * cx)), ax * __fmaf_rn(by, cz, -(bz * cy))));
    float ab = __fmaf_rn(az, bz, __fmaf_rn(ay, by, ax * bx));
    float bc = __fmaf_rn(bz, cz, __fmaf_rn(by, cy, bx * cx));
    float ca = __fmaf_rn(cz, az, __fmaf_rn(cy, ay, cx * ax));
    float labc = la * lb * lc;
    float denom = __fmaf_rn(ca, lb, __fmaf_rn(bc, la, __fmaf_rn(ab, lc, labc)));
    amb |= (fabsf(det) < kCoplanarRel * labc) && (denom < 0.0f);
    return 2.0f * atan2f(det, denom);
}

// The same formula in FP64 from the FP32 inputs (used only for re-checks).
__device__ __forceinline__ double solid_angle_f64(f3 pf, f3 v0, f3 v1, f3 v2) {
    double px = pf.x, py = pf.y, pz = pf.z;
    double ax = v0.x - px, ay = v0.y - py, az = v0.z - pz;
    double bx = v1.x - px, by = v1.y - py, bz = v1.z - pz;
    double cx = v2.x - px, cy = v2.y - py, cz = v2.z - pz;
    double la = sqrt(ax * ax + ay * ay + az * az);
    double lb = sqrt(bx * bx + by * by + bz * bz);
    double lc = sqrt(cx * cx + cy * cy + cz * cz);
    if (la <= 1e-6 || lb <= 1e-6 || lc <= 1e-6) return 0.0;
    double det = ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx);
    double denom = la * lb * lc + (ax * bx + ay * by + az * bz) * lc + (bx * cx + by * cy + bz * cz) * la +
                   (cx * ax + cy * ay + cz * az) * lb;
    return 2.0 * atan2(det, denom);
}

// x / 3, correctly rounded, without a general division: q = RN(x * RN(1/3)), the exact
// remainder r = x - 3q by one FMA, then RN(q + r * RN(1/3)) (Markstein's correction
// step for division by a constant, IEEE Trans. Computers 1990). The engine checks it
// against the IEEE quotient x / 3.0f for every float input (gbsdf_selftest).
__device__ __forceinline__ float div3_rn(float x) {
    const float r3 = 0.333333343267440796f;  // RN(1/3) = 0x3EAAAAAB
    float q = x * r3;
    float r = __fmaf_rn(-3.0f, q, x);
    // r == 0: q is exact (keeps the sign of -0); q infinite: the quotient is q.
    return (r == 0.0f || !(fabsf(q) < __int_as_float(0x7f800000))) ? q : __fmaf_rn(r, r3, q);
}

// div3_rn for x >= +0 or NaN, without its special cases: for finite x >= +0 the
// remainder is +0 exactly when q is exact (and then q + 0 * RN(1/3) = q), and q is finite,
// so the two agree; the self-test (gbsdf_selftest(0)) checks every finite non-negative
// float.
// The eikonal's 3D candidate s0 + s1 + s2 + root is such an x.
__device__ __forceinline__ float div3_pos(float x) {
    const float r3 = 0.333333343267440796f;  // RN(1/3)
    const float q = x * r3;
    return __fmaf_rn(__fmaf_rn(-3.0f, q, x), r3, q);
}

// The same squared distance in FP64 (Ericson's regions, Real-Time Collision Detection
// 5.1.5), for the band error statement: the point and vertices are the FP32 inputs, every
// operation FP64.
__device__ __forceinline__ double ptd_sq_f64(double px, double py, double pz, const float* v) {
    const double ax = v[0], ay = v[1], az = v[2], bx = v[3], by = v[4], bz = v[5], cx = v[6], cy = v[7], cz = v[8];
    const double abx = bx - ax, aby = by - ay, abz = bz - az, acx = cx - ax, acy = cy - ay, acz = cz - az;
    const double apx = px - ax, apy = py - ay, apz = pz - az;
    auto d2 = [](double x, double y, double z) { return x * x + y * y + z * z; };
    const double d1 = abx * apx + aby * apy + abz * apz, d2v = acx * apx + acy * apy + acz * apz;
    if (d1 <= 0.0 && d2v <= 0.0) return d2(apx, apy, apz);
    const double bpx = px - bx, bpy = py - by, bpz = pz - bz;
    const double d3 = abx * bpx + aby * bpy + abz * bpz, d4 = acx * bpx + acy * bpy + acz * bpz;
    if (d3 >= 0.0 && d4 <= d3) return d2(bpx, bpy, bpz);
    const double vc = d1 * d4 - d3 * d2v;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        const double t = d1 / (d1 - d3);
        return d2(px - (ax + t * abx), py - (ay + t * aby), pz - (az + t * abz));
    }
    const double cpx = px - cx, cpy = py - cy, cpz = pz - cz;
    const double d5 = abx * cpx + aby * cpy + abz * cpz, d6 = acx * cpx + acy * cpy + acz * cpz;
    if (d6 >= 0.0 && d5 <= d6) return d2(cpx, cpy, cpz);
    const double vb = d5 * d2v - d1 * d6;
    if (vb <= 0.0 && d2v >= 0.0 && d6 <= 0.0) {
        const double t = d2v / (d2v - d6);
        return d2(px - (ax + t * acx), py - (ay + t * acy), pz - (az + t * acz));
    }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        const double t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return d2(px - (bx + t * (cx - bx)), py - (by + t * (cy - by)), pz - (bz + t * (cz - bz)));
    }
    const double den = 1.0 / (va + vb + vc);
    const double sv = vb * den, sw = vc * den;
    return d2(px - (ax + abx * sv + acx * sw), py - (ay + aby * sv + acy * sw), pz - (az + abz * sv + acz * sw));
}

// Three-input minimum and maximum (PTX ISA 8.8, sm_100 and later): these equal
// fminf(a, fminf(b, c)) and fmaxf(a, fmaxf(b, c)) exactly (a minimum or maximum rounds
// nothing; without the .NaN modifier a NaN operand is passed over, as by fminf). The x
// pipeline clamps a pair of tile neighbours, either of which may be the tiles' NaN
// out-of-lattice fill, with min3f(a, b, far sentinel); the Godunov updates never see a
// NaN operand.
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Packed FP32 pairs (Blackwell's f32x2 arithmetic, PTX ISA 8.6, sm_100 and later): one
// instruction rounds each lane exactly as the scalar instruction does (round to nearest
// even, subnormals kept), so a pair of independent updates costs half the issue slots
// for every add, subtract, multiply and fused multiply-add.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(f32x2 r, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// The reference's Godunov update, rhi_eikonal_godunov (cuda_rasterizer.cu:405-425),
// operation for operation as the reference's own build computes it: nvcc's default FMA
// contraction fuses disc = fma(2h, h, -(d*d)) (d = s1 - s0) and the halved 3D pairwise
// sum S = fma(e2, e2, fma(e1, e1, d*d)) (e1 = s2 - s1, e2 = s2 - s0); 3h^2 - S/2 keeps
// its roundings. This engine is compiled without contraction, so the fused operations are
// written out. The final division by 3 uses div3_rn, which rounds identically to the IEEE
// quotient. The branches are kept: whole warps skip the 2D / 3D work where the 1D update
// applies.
__device__ __forceinline__ float godunov_ref(float ax, float ay, float az, float h) {
    const float s0 = min3f(ax, ay, az);
    const float s2 = max3f(ax, ay, az);
    const float s1 = ax + ay + az - s0 - s2;
    float updated = s0 + h;
    if (updated > s1) {
        const float d = s1 - s0;
        const float dd = d * d;
        const float disc = __fmaf_rn(2.0f * h, h, -dd);
        if (disc >= 0.0f) {
            updated = (s0 + s1 + sqrtf(disc)) * 0.5f;
            if (updated > s2) {
                const float e1 = s2 - s1, e2 = s2 - s0;
                const float S = __fmaf_rn(e2, e2, __fmaf_rn(e1, e1, dd));
                const float disc3 = 3.0f * h * h - S * 0.5f;
                if (disc3 >= 0.0f) updated = div3_rn(s0 + s1 + s2 + sqrtf(disc3));
            }
        }
    }
    return updated;
}

// godunov_ref with the 1D, 2D and 3D candidates all formed and the reference's branch
// conditions selecting among them (same operands, same roundings). Past the first sweeps
// more than 95% of warp steps hold a lane that needs the 2D update and most hold one that
// needs the 3D update, so branching saves little; without branches the updates of a
// thread's independent lines interleave. A square root whose candidate is not selected
// takes 1 in place of a negative discriminant.
__device__ __forceinline__ float godunov_ref_sel(float ax, float ay, float az, float h) {
    const float s0 = min3f(ax, ay, az);
    const float s2 = max3f(ax, ay, az);
    const float s1 = ax + ay + az - s0 - s2;
    const float u1 = s0 + h;
    const float d = s1 - s0;
    const float dd = d * d;
    const float disc = __fmaf_rn(2.0f * h, h, -dd);
    const float e1 = s2 - s1, e2 = s2 - s0;
    const float disc3 = 3.0f * h * h - __fmaf_rn(e2, e2, __fmaf_rn(e1, e1, dd)) * 0.5f;
    const bool ok2 = disc >= 0.0f, ok3 = disc3 >= 0.0f;
    const float u2 = (s0 + s1 + sqrtf(ok2 ? disc : 1.0f)) * 0.5f;
    const float u3 = div3_rn(s0 + s1 + s2 + sqrtf(ok3 ? disc3 : 1.0f));
    const bool take2 = (u1 > s1) && ok2;
    const bool take3 = take2 && (u2 > s2) && ok3;
    return take3 ? u3 : (take2 ? u2 : u1);
}

// Reciprocal square root approximation (the MUFU unit; relative error below 2^-22.9 per
// the PTX ISA's rsqrt.approx). Subnormal operands flush to zero (the result is +inf):
// nsqrt2_rn only takes zero and normal operands.
__device__ __forceinline__ float rsqrt_approx(float a) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// -sqrt(a) in both lanes of NA = -a, correctly rounded (bit-identical to -sqrtf(a)) for
// every a in [2^-100, 2^100], and a zero of either sign for a = 0 (NA = +0 or -0). Markstein's FMA square root (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): y ~ 1/sqrt(a), g = a*y, h = y/2; one Newton step on h,
// r = 1/2 - g*h, h1 = h + h*r; the residual e = g*g - a, exact in one FMA; sqrt(a) =
// g - e*h1. It runs on the negated values: rounding to nearest is symmetric, so each step
// is the exact negation of the positive form. y is capped at 2^100 so that a = 0 gives 0.
// A lane with a < 0 gives a meaningless value. Below 2^-100 the residual e can underflow
// (roots of operands under 2^-102 misround); pair_sqrt_ok keeps the updates' operands out
// of that range. The self-test (gbsdf_selftest(0)) checks zero and every float in
// [2^-100, 2^100] against sqrtf.
__device__ __forceinline__ f32x2 nsqrt2_rn(f32x2 NA, f32x2 half) {
    float na0, na1;
    up2(NA, na0, na1);
    const f32x2 Y = pk2(fminf(rsqrt_approx(fabsf(na0)), 0x1p100f), fminf(rsqrt_approx(fabsf(na1)), 0x1p100f));
    const f32x2 NG = mul2(NA, Y);
    const f32x2 H = mul2(Y, half);
    const f32x2 H1 = fma2(H, fma2(NG, H, half), H);
    return fma2(fma2(NG, NG, NA), H1, NG);
}

// nsqrt2_rn for one value: the same operations on scalars.
__device__ __forceinline__ float nsqrt_rn(float na) {
    const float y = fminf(rsqrt_approx(fabsf(na)), 0x1p100f);
    const float ng = na * y, hh = y * 0.5f;
    const float h1 = __fmaf_rn(hh, __fmaf_rn(ng, hh, 0.5f), hh);
    return __fmaf_rn(__fmaf_rn(ng, ng, na), h1, ng);
}

// godunov_ref without branches and with nsqrt_rn for the square roots (the roundings of
// godunov_ref_pair's lanes): the 1D, 2D and 3D candidates are all formed and the
// reference's conditions select one, so no lane waits for another's branch and the 2D
// and 3D arithmetic overlap. m2h = -2h, na3 = -(3.0f * h * h). For voxel sizes with
// pair_sqrt_ok.
__device__ __forceinline__ float godunov_ref_nb(float ax, float ay, float az, float h, float m2h, float na3) {
    const float s0 = min3f(ax, ay, az), s2 = max3f(ax, ay, az);
    const float s1 = ax + ay + az - s0 - s2;
    const float u1 = s0 + h;
    const float d = s1 - s0;
    const float dd = d * d;
    const float nd = __fmaf_rn(m2h, h, dd);  // -disc
    const float e1 = s2 - s1, e2 = s2 - s0;
    const float nd3 = __fmaf_rn(__fmaf_rn(e2, e2, __fmaf_rn(e1, e1, dd)), 0.5f, na3);  // -disc3
    const float t01 = s0 + s1;
    const float u2 = (t01 - nsqrt_rn(nd)) * 0.5f;
    const float u3 = div3_pos((t01 + s2) - nsqrt_rn(nd3));
    const bool t2 = (u1 > s1) && (nd <= 0.0f);
    const bool t3 = t2 && (u2 > s2) && (nd3 <= 0.0f);
    return t3 ? u3 : (t2 ? u2 : u1);
}

// Constants of godunov_ref_nbp for one voxel size.
struct GodunovOneConsts {
    float h, m2h, na3, r3;
    f32x2 half, half_r3;  // (1/2, 1/2), (1/2, RN(1/3))
};
__device__ __forceinline__ GodunovOneConsts godunov_one_consts(float h) {
    const float r3 = 0.333333343267440796f;
    return GodunovOneConsts{h, -2.0f * h, -(3.0f * h * h), r3, pk2(0.5f, 0.5f), pk2(0.5f, r3)};
}

// godunov_ref_nb for one voxel with the operations of its 2D and 3D candidates paired on
// packed FP32 lanes where they are independent: (d, e2) = (s1 - s0, s2 - s0), the two
// square roots in one nsqrt2_rn, (t01 - r2, t012 - r3) and (x2 / 2, x3 * RN(1/3)). Each lane
// is the scalar operation of godunov_ref_nb on the same operands, so the result is the same
// bit for bit. For a serial chain (the x sweep's one line per thread), where no second
// voxel is at hand to pair with. Voxel sizes with pair_sqrt_ok.
__device__ __forceinline__ float godunov_ref_nbp(float ax, float ay, float az, const GodunovOneConsts& c) {
    const float s0 = min3f(ax, ay, az), s2 = max3f(ax, ay, az);
    const float s1 = ax + ay + az - s0 - s2;
    const float u1 = s0 + c.h;
    float d, e2;
    up2(sub2(pk2(s1, s2), pk2(s0, s0)), d, e2);
    const float dd = d * d;
    const float nd = __fmaf_rn(c.m2h, c.h, dd);  // -disc
    const float e1 = s2 - s1;
    const float nd3 = __fmaf_rn(__fmaf_rn(e2, e2, __fmaf_rn(e1, e1, dd)), 0.5f, c.na3);  // -disc3
    const float t01 = s0 + s1;
    const f32x2 X = sub2(pk2(t01, t01 + s2), nsqrt2_rn(pk2(nd, nd3), c.half));  // (t01 + r2, t012 + r3)
    float u2, q, x3;
    up2(mul2(X, c.half_r3), u2, q);
    {
        float x2;
        up2(X, x2, x3);
    }
    const float u3 = __fmaf_rn(__fmaf_rn(-3.0f, q, x3), c.r3, q);  // div3_pos(x3)
    const bool t2 = (u1 > s1) && (nd <= 0.0f);
    const bool t3 = t2 && (u2 > s2) && (nd3 <= 0.0f);
    return t3 ? u3 : (t2 ? u2 : u1);
}

// Voxel sizes for which every square-root operand of the paired updates lies in
// nsqrt2_rn's checked range, {0} and [2^-100, 2^100]: a non-zero discriminant
// 2h*h - d*d is at least 2^(2e-45) with e = floor(log2 h) (the granularity of the exact
// product), i.e. at least 2^-85 for h >= 2^-20, and no operand exceeds 3h^2 < 2^42 for
// h <= 2^20; a non-zero 3D discriminant 3h^2 - S/2 is either near 3h^2 or, where S/2 is
// near 3h^2, a multiple of ulp(3h^2)/2 >= 2^-64. Other voxel sizes take the scalar kernels.
__host__ __device__ __forceinline__ bool pair_sqrt_ok(float h) { return h >= 0x1p-20f && h <= 0x1p20f; }

// Constants of godunov_ref_pair for one voxel size, each in both lanes.
struct GodunovPairConsts {
    f32x2 h, m2h, na3, half, r3, m3;
};
__device__ __forceinline__ GodunovPairConsts godunov_pair_consts(float h) {
    const float a3 = 3.0f * h * h;
    return GodunovPairConsts{pk2(h, h),       pk2(-2.0f * h, -2.0f * h), pk2(-a3, -a3),
                             pk2(0.5f, 0.5f), pk2(0.333333343267440796f, 0.333333343267440796f),
                             pk2(-3.0f, -3.0f)};
}

// godunov_ref_sel for two independent voxels at once: the arithmetic on packed pairs,
// the ordering and selections per lane. Every value rounds exactly as in godunov_ref_sel,
// formed negated where that saves an operation (rounding to nearest is symmetric):
// -disc = fma(-2h, h, dd); -disc3 = fma(S, 1/2, -3h^2), one rounding of the exact
// S/2 - 3h^2 where the reference rounds S*0.5 (exact) and then 3h^2 - S*0.5; the square
// roots are nsqrt2_rn (correctly rounded, as sqrtf); the division by 3 is div3_pos. A
// candidate whose discriminant is negative holds a meaningless value and is not selected.
__device__ __forceinline__ void godunov_ref_pair(float ax0, float ay0, float az0, float ax1, float ay1, float az1,
                                                 const GodunovPairConsts& c, float& out0, float& out1) {
    const float s00 = min3f(ax0, ay0, az0), s20 = max3f(ax0, ay0, az0);
    const float s01 = min3f(ax1, ay1, az1), s21 = max3f(ax1, ay1, az1);
    const f32x2 S0 = pk2(s00, s01), S2 = pk2(s20, s21);
    const f32x2 S1 = sub2(sub2(add2(add2(pk2(ax0, ax1), pk2(ay0, ay1)), pk2(az0, az1)), S0), S2);
    const f32x2 U1 = add2(S0, c.h);
    const f32x2 D = sub2(S1, S0);
    const f32x2 DD = mul2(D, D);
    const f32x2 ND = fma2(c.m2h, c.h, DD);  // -disc
    const f32x2 E2 = sub2(S2, S0), E1 = sub2(S2, S1);
    const f32x2 SS = fma2(E2, E2, fma2(E1, E1, DD));
    const f32x2 ND3 = fma2(SS, c.half, c.na3);  // -disc3
    float nd0, nd1, nd30, nd31;
    up2(ND, nd0, nd1);
    up2(ND3, nd30, nd31);
    const bool ok20 = nd0 <= 0.0f, ok21 = nd1 <= 0.0f, ok30 = nd30 <= 0.0f, ok31 = nd31 <= 0.0f;
    const f32x2 T01 = add2(S0, S1);
    const f32x2 U2 = mul2(sub2(T01, nsqrt2_rn(ND, c.half)), c.half);
    const f32x2 X3 = sub2(add2(T01, S2), nsqrt2_rn(ND3, c.half));
    const f32x2 Q = mul2(X3, c.r3);
    const f32x2 U3 = fma2(fma2(c.m3, Q, X3), c.r3, Q);
    float u10, u11, s10, s11, u20, u21, u30, u31;
    up2(U1, u10, u11);
    up2(S1, s10, s11);
    up2(U2, u20, u21);
    up2(U3, u30, u31);
    const bool t20 = (u10 > s10) && ok20, t21 = (u11 > s11) && ok21;
    const bool t30 = t20 && (u20 > s20) && ok30, t31 = t21 && (u21 > s21) && ok31;
    out0 = t30 ? u30 : (t20 ? u20 : u10);
    out1 = t31 ? u31 : (t21 ? u21 : u11);
}

// Corrected, monotone Godunov update (the engine's exact mode): sorted minima,
// true 3D discriminant 3h^2 - sum_{i<j}(s_i - s_j)^2, increments formed from
// differences and added to the smallest neighbour once.
__device__ __forceinline__ float godunov_exact(float a, float b, float c, float h) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    const float s0 = fminf(lo, c);
    const float m = fmaxf(lo, c);
    const float s1 = fminf(m, hi);
    const float s2 = fmaxf(m, hi);
    float u = s0 + h;
    if (u > s1) {
        const float d1 = s1 - s0;
        const float disc = 2.0f * h * h - d1 * d1;
        u = s0 + (d1 + sqrtf(fmaxf(disc, 0.0f))) * 0.5f;
        if (u > s2) {
            const float d2 = s2 - s0;
            const float e = s2 - s1;
            const float disc3 = 3.0f * h * h - (d1 * d1 + e * e + d2 * d2);
            u = s0 + div3_rn(d1 + d2 + sqrtf(fmaxf(disc3, 0.0f)));
        }
    }
    return u;
}

template <int RULE>
__device__ __forceinline__ float godunov(float ax, float ay, float az, float h) {
    if constexpr (RULE == 0) return godunov_ref(ax, ay, az, h);
    else return godunov_exact(ax, ay, az, h);
}

// The same updates for kernels that interleave several lines per thread.
template <int RULE>
__device__ __forceinline__ float godunov_sel(float ax, float ay, float az, float h) {
    if constexpr (RULE == 0) return godunov_ref_sel(ax, ay, az, h);
    else return godunov_exact(ax, ay, az, h);
}

// Voxel lattice point, as the reference forms it: (min + i) * h in FP32.
__device__ __forceinline__ f3 lattice_point(int mnx, int mny, int mnz, int x, int y, int z, float h) {
    return f3{(float)(mnx + x) * h, (float)(mny + y) * h, (float)(mnz + z) * h};
}

}  // namespace gbsdf
