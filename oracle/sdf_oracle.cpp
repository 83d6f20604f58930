// SPDX-License-Identifier: MIT
//
// oracle/sdf_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// The CPU oracle for the mesh-to-SDF path. Only tests/, the smoke check in
// __graft_entry__.py and bench.py's CPU-baseline / reference arm load this
// library; the product (rhizome_v24.15_gb300/csrc) never links or calls it.
//
// It restates, stage by stage, the reference's "fast SDF" path
//   native/src/engine/sdf/cuda_rasterizer.cu  (RAST)
//     [init] gpu_fill_float_kernel              RAST:194-203
//     [A]    gpu_splat_band_distances_kernel    RAST:211-268
//     [B]    host CSR + parity columns          RAST:824-882, RAST:279-368
//     [C]    gpu_exact_winding_fixup_kernel     RAST:374-400
//     [D]    rhi_eikonal_godunov + FSM sweeps   RAST:405-513, loop RAST:987-1064
//     [D2/3] sentinel audit / clamp             RAST:523-556
//     [E]    verify samples + patch boxes       RAST:566-646, loop RAST:1078-1132
//     [F]    sign apply                         RAST:650-661
//   the legacy exact kernel mesh_to_sdf_kernel  RAST:97-185 (+ tile headers RAST:1197-1235)
//   the build_from_mesh front-end               RAST:1340-1435, MATH:484-514
// and the geometry primitives of native/src/core/math_utils.cuh (MATH:43-132).
//
// Floating point: compiled with -ffp-contract=off, so every product and sum
// rounds once, in the source order of the reference expressions, on x86 and
// on aarch64 alike. The GPU kernels of the product use the same evaluation
// order without contraction where results must match bit for bit.
//
// Deliberate, documented differences from the reference GPU code:
//  * FSM sweeps use lockstep semantics: all lines of one sweep read their
//    neighbour lines as they were when the sweep began (the deterministic model
//    of the reference launching every line of a sweep at once, RAST:992-1002;
//    the reference's own lines race, RAST:427-432). The reference's update
//    (RAST:405-425) is not monotone -- its 3D discriminant halves the pairwise
//    sum (RAST:418) -- so its fixed point depends on the schedule; the schedule
//    is therefore part of the definition and is reproduced exactly.
//  * fsm_mode 2 replaces the update with the corrected, monotone one, whose
//    fixed point is unique (the exact mode of the product).
//  * gwn_mode 1 decides every winding sign exactly (FP32 compensated sum,
//    FP64 re-evaluation when | |w|-0.5 | < 0.05); gwn_mode 0 is the
//    reference's plain FP32 index-order sum.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
};
struct OTri {  // layout of CudaTriangle (cuda_types.hpp:18-21): v0, v1, v2, normal
    V3 v0, v1, v2, n;
};
static_assert(sizeof(OTri) == 48, "CudaTriangle is 48 bytes");

inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// glm::dot(vec3) = (x*x' + y*y') + z*z'
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ---- constants of the reference path (RAST:74-82, RAST:825, RAST:1010, RAST:1027, RAST:298-299)
constexpr size_t kFastMinVoxels = 32ull * 1024ull * 1024ull;
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

// ---- threading helpers -------------------------------------------------------------
template <class F>
void parallel_dyn(long long n, long long grain, int threads, F&& f) {
    if (n <= 0) return;
    if (threads <= 1 || n <= grain) {
        f(0LL, n);
        return;
    }
    std::atomic<long long> next(0);
    auto worker = [&]() {
        for (;;) {
            long long b = next.fetch_add(grain);
            if (b >= n) break;
            f(b, std::min(n, b + grain));
        }
    };
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
}

}  // namespace

// =====================================================================================
// Geometry primitives (MATH:43-132), restated in the reference's operation order.
// =====================================================================================
static float ptd_sq(V3 p, V3 a, V3 b, V3 c) {
    // point_triangle_distance_sq, MATH:43-106 (Ericson, 7 Voronoi regions)
    V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return dot(ap, ap);
    V3 bp = sub(p, b);
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return dot(bp, bp);
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        V3 cl = add(a, mul(ab, v));
        V3 df = sub(p, cl);
        return dot(df, df);
    }
    V3 cp = sub(p, c);
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return dot(cp, cp);
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        V3 cl = add(a, mul(ac, w));
        V3 df = sub(p, cl);
        return dot(df, df);
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        V3 cl = add(b, mul(sub(c, b), w));
        V3 df = sub(p, cl);
        return dot(df, df);
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    V3 cl = add(add(a, mul(ab, v)), mul(ac, w));
    V3 df = sub(p, cl);
    return dot(df, df);
}

static float solid_angle_f(V3 p, V3 v0, V3 v1, V3 v2) {
    // triangle_solid_angle, MATH:109-132 (Van Oosterom-Strackee)
    V3 a = sub(v0, p), b = sub(v1, p), c = sub(v2, p);
    float la = std::sqrt(dot(a, a)), lb = std::sqrt(dot(b, b)), lc = std::sqrt(dot(c, c));
    if (la <= 1e-6f || lb <= 1e-6f || lc <= 1e-6f) return 0.0f;
    float det = a.x * (b.y * c.z - b.z * c.y) - a.y * (b.x * c.z - b.z * c.x) +
                a.z * (b.x * c.y - b.y * c.x);
    float denom = la * lb * lc + dot(a, b) * lc + dot(b, c) * la + dot(c, a) * lb;
    return 2.0f * std::atan2(det, denom);
}

static double solid_angle_d(V3 pf, V3 v0, V3 v1, V3 v2) {
    // The same formula evaluated in FP64 from the FP32 inputs.
    double px = pf.x, py = pf.y, pz = pf.z;
    double ax = v0.x - px, ay = v0.y - py, az = v0.z - pz;
    double bx = v1.x - px, by = v1.y - py, bz = v1.z - pz;
    double cx = v2.x - px, cy = v2.y - py, cz = v2.z - pz;
    double la = std::sqrt(ax * ax + ay * ay + az * az);
    double lb = std::sqrt(bx * bx + by * by + bz * bz);
    double lc = std::sqrt(cx * cx + cy * cy + cz * cz);
    if (la <= 1e-6 || lb <= 1e-6 || lc <= 1e-6) return 0.0;
    double det = ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx);
    double denom = la * lb * lc + (ax * bx + ay * by + az * bz) * lc +
                   (bx * cx + by * cy + bz * cz) * la + (cx * ax + cy * ay + cz * az) * lb;
    return 2.0 * std::atan2(det, denom);
}

// Winding-number sign of one lattice point.
//   mode 0: reference, FP32 naive sum in index order (RAST:392-397)
//   mode 1: exact decision. A point whose band distance is <= 1e-5 voxel lies on the
//           surface, where the winding number is 0.5 in exact arithmetic: inside
//           (|w| >= 0.5). Otherwise an FP32 compensated sum decides, unless |w| is
//           within 0.05 of 0.5 or some triangle's term has an uncertain sign (the point
//           nearly coplanar with it and projecting inside it); then FP64 decides.
struct GwnCounters {
    std::atomic<long long> fp64_rechecks{0};
};
constexpr float kSurfaceTolVoxels = 1e-5f;
constexpr float kCoplanarRel = 1e-4f;
static bool gwn_inside(const OTri* tris, int T, V3 p, int mode, GwnCounters* ctr, float dvox, float h,
                       float surface_tol = kSurfaceTolVoxels) {
    if (mode == 0) {
        float s = 0.0f;
        for (int t = 0; t < T; ++t) s += solid_angle_f(p, tris[t].v0, tris[t].v1, tris[t].v2);
        float w = s * kInv4Pi;
        return std::fabs(w) >= 0.5f;
    }
    if (dvox <= surface_tol * h) return true;
    float s = 0.0f, comp = 0.0f;
    bool amb = false;
    for (int t = 0; t < T; ++t) {
        V3 a = sub(tris[t].v0, p), b = sub(tris[t].v1, p), c = sub(tris[t].v2, p);
        float la = std::sqrt(dot(a, a)), lb = std::sqrt(dot(b, b)), lc = std::sqrt(dot(c, c));
        float om = 0.0f;
        if (!(la <= 1e-6f || lb <= 1e-6f || lc <= 1e-6f)) {
            float det = a.x * (b.y * c.z - b.z * c.y) - a.y * (b.x * c.z - b.z * c.x) + a.z * (b.x * c.y - b.y * c.x);
            float denom = la * lb * lc + dot(a, b) * lc + dot(b, c) * la + dot(c, a) * lb;
            if (std::fabs(det) < kCoplanarRel * (la * lb * lc) && denom < 0.0f) amb = true;
            om = 2.0f * std::atan2(det, denom);
        }
        float y = om - comp;
        float u = s + y;
        comp = (u - s) - y;
        s = u;
    }
    float w = s * kInv4Pi;
    if (!amb && std::fabs(std::fabs(w) - 0.5f) >= 0.05f) return std::fabs(w) >= 0.5f;
    if (ctr) ctr->fp64_rechecks.fetch_add(1);
    double sd = 0.0;
    for (int t = 0; t < T; ++t) sd += solid_angle_d(p, tris[t].v0, tris[t].v1, tris[t].v2);
    double wd = sd / (4.0 * 3.14159265358979323846);
    return std::fabs(wd) >= 0.5;
}

static double gwn_value_d(const OTri* tris, int T, V3 p) {
    double sd = 0.0;
    for (int t = 0; t < T; ++t) sd += solid_angle_d(p, tris[t].v0, tris[t].v1, tris[t].v2);
    return sd / (4.0 * 3.14159265358979323846);
}

// Godunov update, RAST:405-425, with the roundings the reference's own build gives it.
// nvcc compiles the reference with its default FMA contraction (native/CMakeLists.txt
// sets no -fmad flag), which fuses two of the products into their sums inside the sweep
// kernel: disc = fma(2h, h, -(d*d)) with d = s1 - s0, and the 3D pairwise sum
// S = fma(e2, e2, fma(e1, e1, d*d)) with e1 = s2 - s1, e2 = s2 - s0; 3h^2 - S/2 keeps
// separate roundings (3h*h is formed once per thread). Pinned bit for bit against the
// reference's gpu_eikonal_fsm_sweep_kernel compiled with its own flags, on sweeps whose
// cross-line neighbours cannot change (tests/test_gpu_reference_gpu.py). std::fma rounds
// once on every host, so the restatement is exact on x86 and Arm alike.
static inline float godunov(float ax, float ay, float az, float h) {
    float s0 = std::fmin(ax, std::fmin(ay, az));
    float s2 = std::fmax(ax, std::fmax(ay, az));
    float s1 = ax + ay + az - s0 - s2;
    float updated = s0 + h;
    if (updated > s1) {
        const float d = s1 - s0;
        const float dd = d * d;
        float disc = std::fma(2.0f * h, h, -dd);
        if (disc >= 0.0f) {
            updated = (s0 + s1 + std::sqrt(disc)) * 0.5f;
            if (updated > s2) {
                const float e1 = s2 - s1, e2 = s2 - s0;
                const float S = std::fma(e2, e2, std::fma(e1, e1, dd));
                float disc3 = 3.0f * h * h - S * 0.5f;
                if (disc3 >= 0.0f) updated = (s0 + s1 + s2 + std::sqrt(disc3)) / 3.0f;
            }
        }
    }
    return updated;
}

// Corrected Godunov update (not in the reference): sorted minima and the true 3D
// discriminant 3h^2 - sum_{i<j}(s_i - s_j)^2. The reference multiplies that pairwise
// sum by 0.5 (RAST:418), which makes its update non-monotone, so its fixed point
// depends on the sweep schedule; this update is monotone and its fixed point is
// unique. The increments are formed from differences (exact when the minima are
// within a factor of two, Sterbenz) and added to s0 once, which keeps FP32 rounding
// to one addition per update.
template <class T>
static inline T godunov_exact_t(T a, T b, T c, T h) {
    if (a > b) std::swap(a, b);
    if (b > c) std::swap(b, c);
    if (a > b) std::swap(a, b);
    T u = a + h;
    if (u > b) {
        T d1 = b - a;
        T disc = T(2) * h * h - d1 * d1;
        T inc = (d1 + std::sqrt(std::max(disc, T(0)))) * T(0.5);
        u = a + inc;
        if (u > c) {
            T d2 = c - a;
            T e = c - b;
            T disc3 = T(3) * h * h - (d1 * d1 + e * e + d2 * d2);
            T inc3 = (d1 + d2 + std::sqrt(std::max(disc3, T(0)))) / T(3);
            u = a + inc3;
        }
    }
    return u;
}
static float godunov_exact_f(float a, float b, float c, float h) { return godunov_exact_t<float>(a, b, c, h); }
static double godunov_exact_d(double a, double b, double c, double h) { return godunov_exact_t<double>(a, b, c, h); }

// =====================================================================================
// Public API (extern "C"): plain pointers and sizes only.
// =====================================================================================
extern "C" {

struct orc_fast_params {
    int fsm_mode;        // 0: reference loop (<= 8 rounds, audit-gated <= 16 extra); 1/2: to convergence
    int gwn_mode;        // 0: reference FP32 naive sum; 1: exact decision
    int threads;         // host threads
    int max_conv_rounds; // cap for fsm_mode 1 (safety only)
    int skip_verify;     // 1: skip stage [E] (used to time/compare stages separately)
    int signed_parity;   // 1: exact signs -- signed crossings, near-lattice rays, surface tolerance 1e-3 voxel
    int skip_eikonal;    // 1: signs and statuses only -- no stage [D]; out_dist holds the signed band field
    int lazy_winding;    // 1: voxels that [C] and the patch boxes would decide by the winding number are
                         //    marked (sign 3), not summed; the probes skip them, since a probe there makes
                         //    the same winding decision as the fixup
};
// Exact-signs mode: voxels within this many voxels of the surface are on it (inside).
constexpr float kSurfaceTolExact = 1e-3f;

struct orc_fast_stats {
    int status;  // 0 ok, 1 invalid input, 2 int-range guard, 3 CSR guard, 4 verify diverged
    int unknown_columns;
    long long fixup_voxels;
    int eikonal_rounds;
    int extra_rounds;
    long long far_residual;
    long long safe_clamped;
    int probes;
    int sites;
    int patch_rounds;
    long long patched_voxels;
    long long fp64_rechecks;
    long long band_voxels;
    double ms_splat, ms_parity, ms_fixup, ms_eikonal, ms_verify, ms_apply, ms_total;
};

float orc_point_triangle_distance_sq(const float* p, const float* a, const float* b, const float* c) {
    return ptd_sq({p[0], p[1], p[2]}, {a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]});
}
float orc_triangle_solid_angle(const float* p, const float* a, const float* b, const float* c) {
    return solid_angle_f({p[0], p[1], p[2]}, {a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]});
}
double orc_triangle_solid_angle_f64(const float* p, const float* a, const float* b, const float* c) {
    return solid_angle_d({p[0], p[1], p[2]}, {a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]});
}
float orc_godunov(float ax, float ay, float az, float h) { return godunov(ax, ay, az, h); }

// Batch forms used to pin the primitives against golden vectors.
void orc_ptd_batch(const float* pts, const float* tris9, long long n, float* out) {
    for (long long i = 0; i < n; ++i)
        out[i] = orc_point_triangle_distance_sq(pts + 3 * i, tris9 + 9 * i, tris9 + 9 * i + 3, tris9 + 9 * i + 6);
}
void orc_solid_angle_batch(const float* pts, const float* tris9, long long n, float* out) {
    for (long long i = 0; i < n; ++i)
        out[i] = orc_triangle_solid_angle(pts + 3 * i, tris9 + 9 * i, tris9 + 9 * i + 3, tris9 + 9 * i + 6);
}

// Generalized winding number at arbitrary points, FP64 (the full-GWN oracle).
void orc_gwn_points_f64(const void* tris_, int T, const float* pts, long long n, double* out_w, int threads) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    parallel_dyn(n, 64, threads, [&](long long b, long long e) {
        for (long long i = b; i < e; ++i) out_w[i] = gwn_value_d(tris, T, {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    });
}

// Exact winding sign (|w| >= 0.5) of listed lattice voxels; mode as gwn_inside.
void orc_gwn_sign_voxels(const void* tris_, int T, float h, const int* mn, const int* dims,
                         const long long* vidx, long long n, int mode, uint8_t* out_inside, int threads) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    long long dx = dims[0], dy = dims[1];
    parallel_dyn(n, 16, threads, [&](long long b, long long e) {
        for (long long i = b; i < e; ++i) {
            long long v = vidx[i];
            int x = (int)(v % dx), y = (int)((v / dx) % dy), z = (int)(v / (dx * dy));
            V3 p{(float)(mn[0] + x) * h, (float)(mn[1] + y) * h, (float)(mn[2] + z) * h};
            out_inside[i] = gwn_inside(tris, T, p, mode, nullptr, 1e30f, h) ? 1 : 0;
        }
    });
}

// ---- [init] + [A] band splat (RAST:194-203, RAST:211-268) ---------------------------
// Threads own disjoint z-layers; each layer visits every triangle exactly as one
// reference thread (triangle, z) does, so the result is the same min over the same
// candidate set. Returns the number of band voxels (< sentinel).
long long orc_splat_band(const void* tris_, int T, float h, const int* mn, const int* dims, float* dist,
                         int threads) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    const size_t N = (size_t)dx * dy * dz;
    for (size_t i = 0; i < N; ++i) dist[i] = kFarSentinel;
    const float bw = (float)kBandVoxels * h;
    const float band_sq = bw * bw;
    std::vector<float> bb((size_t)T * 6);
    for (int t = 0; t < T; ++t) {
        const OTri& tr = tris[t];
        float* o = &bb[(size_t)t * 6];
        o[0] = std::fmin(tr.v0.x, std::fmin(tr.v1.x, tr.v2.x));
        o[1] = std::fmax(tr.v0.x, std::fmax(tr.v1.x, tr.v2.x));
        o[2] = std::fmin(tr.v0.y, std::fmin(tr.v1.y, tr.v2.y));
        o[3] = std::fmax(tr.v0.y, std::fmax(tr.v1.y, tr.v2.y));
        o[4] = std::fmin(tr.v0.z, std::fmin(tr.v1.z, tr.v2.z));
        o[5] = std::fmax(tr.v0.z, std::fmax(tr.v1.z, tr.v2.z));
    }
    const size_t zstride = (size_t)dy * dx;
    parallel_dyn(dz, 1, threads, [&](long long zb, long long ze) {
        for (long long z = zb; z < ze; ++z) {
            float wz = (float)(mn[2] + (int)z) * h;
            for (int t = 0; t < T; ++t) {
                const float* o = &bb[(size_t)t * 6];
                float tx0 = o[0], tx1 = o[1], ty0 = o[2], ty1 = o[3], tz0 = o[4], tz1 = o[5];
                if (wz < tz0 - bw || wz > tz1 + bw) continue;
                float bdz = (wz < tz0) ? (tz0 - wz) : ((wz > tz1) ? (wz - tz1) : 0.0f);
                int x0 = (int)std::ceil((tx0 - bw) / h) - mn[0];
                int x1 = (int)std::floor((tx1 + bw) / h) - mn[0];
                int y0 = (int)std::ceil((ty0 - bw) / h) - mn[1];
                int y1 = (int)std::floor((ty1 + bw) / h) - mn[1];
                if (x0 < 0) x0 = 0;
                if (y0 < 0) y0 = 0;
                if (x1 > dx - 1) x1 = dx - 1;
                if (y1 > dy - 1) y1 = dy - 1;
                if (x1 < x0 || y1 < y0) continue;
                const OTri& tr = tris[t];
                for (int y = y0; y <= y1; ++y) {
                    float py = (float)(mn[1] + y) * h;
                    float bdy = (py < ty0) ? (ty0 - py) : ((py > ty1) ? (py - ty1) : 0.0f);
                    size_t row = (size_t)z * zstride + (size_t)y * dx;
                    for (int x = x0; x <= x1; ++x) {
                        float px = (float)(mn[0] + x) * h;
                        float bdx = (px < tx0) ? (tx0 - px) : ((px > tx1) ? (px - tx1) : 0.0f);
                        if (bdx * bdx + bdy * bdy + bdz * bdz > band_sq) continue;
                        float d2 = ptd_sq({px, py, wz}, tr.v0, tr.v1, tr.v2);
                        if (d2 <= band_sq) {
                            float d = std::sqrt(d2);
                            if (d < dist[row + x]) dist[row + x] = d;
                        }
                    }
                }
            }
        }
    });
    long long band = 0;
    for (size_t i = 0; i < N; ++i) band += (dist[i] < kFarSentinel) ? 1 : 0;
    return band;
}

// ---- [B] parity signs (RAST:824-882 host CSR, RAST:279-368 kernel) ------------------
// Returns the number of unknown columns, or -1 when the CSR guard declines
// (total_entries <= 0 or > 1e8, RAST:867-869).
// signed = 0: the reference's parity (odd or > 128 crossings -> unknown column).
// signed = 1: signed crossings -- a crossing whose projected triangle is clockwise in xy
// (normal pointing down: entering an outward-oriented solid going up) counts +1, a
// counter-clockwise one -1; the running sum below a voxel is the winding number of a
// closed, consistently oriented mesh (overlapping shells included) and the voxel is
// inside iff it is nonzero. A column whose total is nonzero (a ray through a hole) or
// that overflows is unknown.
// The exact-signs mode casts its rays 1000x closer to the lattice point than the
// reference's jitter (still several float ulps away for |coordinate index| < 4096).
constexpr float kJXExact = 3.7e-4f;
constexpr float kJYExact = 5.1e-4f;
long long orc_parity_signs_mode(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                                int threads, int signed_mode);
long long orc_parity_signs(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                           int threads) {
    return orc_parity_signs_mode(tris_, T, h, mn, dims, sign, threads, 0);
}
long long orc_parity_signs_mode(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                                int threads, int signed_mode) {
    const float jx = signed_mode ? kJXExact : kJX, jy = signed_mode ? kJYExact : kJY;
    const OTri* tris = static_cast<const OTri*>(tris_);
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    const int sdx = (dx + kSup - 1) / kSup, sdy = (dy + kSup - 1) / kSup;
    const size_t nsup = (size_t)sdx * sdy;
    std::vector<float> xyab((size_t)T * 4);
    std::vector<long long> start(nsup + 1, 0);
    std::vector<int> sx0(T), sx1(T), sy0(T), sy1(T);
    long long total = 0;
    for (int t = 0; t < T; ++t) {
        const OTri& tr = tris[t];
        float minx = std::min(tr.v0.x, std::min(tr.v1.x, tr.v2.x));
        float maxx = std::max(tr.v0.x, std::max(tr.v1.x, tr.v2.x));
        float miny = std::min(tr.v0.y, std::min(tr.v1.y, tr.v2.y));
        float maxy = std::max(tr.v0.y, std::max(tr.v1.y, tr.v2.y));
        xyab[4 * (size_t)t + 0] = minx;
        xyab[4 * (size_t)t + 1] = miny;
        xyab[4 * (size_t)t + 2] = maxx;
        xyab[4 * (size_t)t + 3] = maxy;
        int cx0 = (int)std::floor(minx / h) - mn[0] - 1;
        int cx1 = (int)std::ceil(maxx / h) - mn[0] + 1;
        int cy0 = (int)std::floor(miny / h) - mn[1] - 1;
        int cy1 = (int)std::ceil(maxy / h) - mn[1] + 1;
        int a0 = std::max(0, cx0 / kSup), a1 = std::min(sdx - 1, cx1 / kSup);
        int b0 = std::max(0, cy0 / kSup), b1 = std::min(sdy - 1, cy1 / kSup);
        sx0[t] = a0; sx1[t] = a1; sy0[t] = b0; sy1[t] = b1;
        if (a1 < a0 || b1 < b0) continue;
        for (int sy = b0; sy <= b1; ++sy)
            for (int sx = a0; sx <= a1; ++sx) ++start[(size_t)sy * sdx + sx + 1];
        total += (long long)(a1 - a0 + 1) * (b1 - b0 + 1);
    }
    if (total <= 0 || total > 100000000LL) return -1;
    for (size_t i = 1; i <= nsup; ++i) start[i] += start[i - 1];
    std::vector<int> lst((size_t)total);
    {
        std::vector<long long> cur(start.begin(), start.end() - 1);
        for (int t = 0; t < T; ++t)
            for (int sy = sy0[t]; sy <= sy1[t]; ++sy)
                for (int sx = sx0[t]; sx <= sx1[t]; ++sx) lst[(size_t)cur[(size_t)sy * sdx + sx]++] = t;
    }
    const size_t zstride = (size_t)dy * dx;
    std::atomic<long long> unknown(0);
    parallel_dyn((long long)dx * dy, 256, threads, [&](long long cb, long long ce) {
        float hit[kParityMaxHits];
        int hsg[kParityMaxHits];
        long long local_unknown = 0;
        for (long long col = cb; col < ce; ++col) {
            int cx = (int)(col % dx), cy = (int)(col / dx);
            float rx = ((float)(mn[0] + cx) + jx) * h;
            float ry = ((float)(mn[1] + cy) + jy) * h;
            int nh = 0;
            bool bad = false;
            size_t sup = (size_t)(cy >> 2) * sdx + (cx >> 2);
            for (long long e = start[sup]; e < start[sup + 1]; ++e) {
                int ti = lst[(size_t)e];
                const float* ab = &xyab[4 * (size_t)ti];
                if (rx < ab[0] || rx > ab[2] || ry < ab[1] || ry > ab[3]) continue;
                const OTri& tr = tris[ti];
                // the reference's build contracts a*b - c*d to fma(a, b, -(c*d)) and the hit
                // height's sum to fma(d0, z2, fma(d1, z0, d2*z1))
                float d0 = std::fma(tr.v1.x - tr.v0.x, ry - tr.v0.y, -((tr.v1.y - tr.v0.y) * (rx - tr.v0.x)));
                float d1 = std::fma(tr.v2.x - tr.v1.x, ry - tr.v1.y, -((tr.v2.y - tr.v1.y) * (rx - tr.v1.x)));
                float d2 = std::fma(tr.v0.x - tr.v2.x, ry - tr.v2.y, -((tr.v0.y - tr.v2.y) * (rx - tr.v2.x)));
                bool pos = (d0 > 0.0f && d1 > 0.0f && d2 > 0.0f);
                bool neg = (d0 < 0.0f && d1 < 0.0f && d2 < 0.0f);
                if (!pos && !neg) continue;
                float area2 = d0 + d1 + d2;
                if (std::fabs(area2) < 1e-12f) continue;
                float zh = std::fma(d0, tr.v2.z, std::fma(d1, tr.v0.z, d2 * tr.v1.z)) / area2;
                if (nh < kParityMaxHits) {
                    hsg[nh] = neg ? 1 : -1;
                    hit[nh++] = zh;
                } else {
                    bad = true;
                    break;
                }
            }
            size_t base = (size_t)cy * dx + cx;
            int total = 0;
            for (int i = 0; i < nh; ++i) total += hsg[i];
            if (bad || (signed_mode ? (total != 0) : (nh & 1))) {
                for (int z = 0; z < dz; ++z) sign[(size_t)z * zstride + base] = 2;
                ++local_unknown;
                continue;
            }
            // insertion sort of (height, sign) pairs by height
            for (int i = 1; i < nh; ++i) {
                float key = hit[i];
                int ks = hsg[i];
                int j = i - 1;
                while (j >= 0 && hit[j] > key) {
                    hit[j + 1] = hit[j];
                    hsg[j + 1] = hsg[j];
                    --j;
                }
                hit[j + 1] = key;
                hsg[j + 1] = ks;
            }
            int k = 0;
            bool inside = false;
            int wnum = 0;
            for (int z = 0; z < dz; ++z) {
                float zc = (float)(mn[2] + z) * h;
                while (k < nh && hit[k] < zc) {
                    inside = !inside;
                    wnum += hsg[k];
                    ++k;
                }
                sign[(size_t)z * zstride + base] = (signed_mode ? (wnum != 0) : inside) ? 1 : 0;
            }
        }
        unknown.fetch_add(local_unknown);
    });
    return unknown.load();
}

// ---- [C] exact winding fixup (RAST:374-400): every sign==2 voxel -----------------------
long long orc_fixup_unknown_tol(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                                const float* dist, int gwn_mode, int threads, long long* fp64_rechecks, float tol);
long long orc_fixup_unknown(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                            const float* dist, int gwn_mode, int threads, long long* fp64_rechecks) {
    return orc_fixup_unknown_tol(tris_, T, h, mn, dims, sign, dist, gwn_mode, threads, fp64_rechecks,
                                 kSurfaceTolVoxels);
}
long long orc_fixup_unknown_tol(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                                const float* dist, int gwn_mode, int threads, long long* fp64_rechecks, float tol) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    const long long dx = dims[0], dy = dims[1], dz = dims[2];
    const long long N = dx * dy * dz;
    std::vector<long long> todo;
    for (long long i = 0; i < N; ++i)
        if (sign[i] == 2) todo.push_back(i);
    GwnCounters ctr;
    parallel_dyn((long long)todo.size(), 8, threads, [&](long long b, long long e) {
        for (long long k = b; k < e; ++k) {
            long long i = todo[(size_t)k];
            int x = (int)(i % dx), y = (int)((i / dx) % dy), z = (int)(i / (dx * dy));
            V3 p{(float)(mn[0] + x) * h, (float)(mn[1] + y) * h, (float)(mn[2] + z) * h};
            sign[i] = gwn_inside(tris, T, p, gwn_mode, &ctr, dist ? dist[i] : 1e30f, h, tol) ? 1 : 0;
        }
    });
    if (fp64_rechecks) *fp64_rechecks += ctr.fp64_rechecks.load();
    return (long long)todo.size();
}

// ---- [D] one directional FSM sweep (RAST:433-513) ------------------------------------
// Lockstep semantics: every line of the sweep reads its neighbour lines as they were
// when the sweep started (the reference launches all lines of a sweep concurrently,
// RAST:992-1002; lockstep is the deterministic model of that launch), while the
// swept line itself is walked sequentially in place. Deterministic for any thread
// count. rule 0 = the reference's update (rhi_eikonal_godunov); rule 1 = the
// corrected, monotone update (godunov_exact).
int orc_fsm_sweep_rule(float* g, const int* dims, float h, int axis, int dir, int rule, int threads) {
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    const long long sx = 1, sy = dx, sz = (long long)dx * dy;
    const size_t N = (size_t)dx * dy * dz;
    std::vector<float> snap(g, g + N);
    const float* s0 = snap.data();
    int n[3] = {dx, dy, dz};
    int a1 = (axis == 0) ? 1 : 0;  // first cross axis
    int a2 = (axis == 2) ? 1 : 2;  // second cross axis
    long long st[3] = {sx, sy, sz};
    const long long sa = st[axis];
    std::atomic<int> changed(0);
    long long nl = (long long)n[a1] * n[a2];
    parallel_dyn(nl, 64, threads, [&](long long b, long long e) {
        int local = 0;
        for (long long li = b; li < e; ++li) {
            int c[3];
            c[a1] = (int)(li % n[a1]);
            c[a2] = (int)(li / n[a1]);
            float prev = kFarSentinel;  // new value of the upstream neighbour on this line
            for (int s = 0; s < n[axis]; ++s) {
                c[axis] = (dir > 0) ? s : (n[axis] - 1 - s);
                long long idx = c[0] * sx + c[1] * sy + (long long)c[2] * sz;
                float cur = s0[idx];
                float nb[3];
                for (int k = 0; k < 3; ++k) {
                    long long stk = st[k];
                    float lo = (c[k] > 0) ? s0[idx - stk] : kFarSentinel;
                    float hi = (c[k] < n[k] - 1) ? s0[idx + stk] : kFarSentinel;
                    if (k == axis) {  // upstream neighbour comes from this sweep
                        if (dir > 0) lo = (c[k] > 0) ? prev : kFarSentinel;
                        else hi = (c[k] < n[k] - 1) ? prev : kFarSentinel;
                    }
                    nb[k] = std::fmin(lo, hi);
                }
                float upd = rule ? godunov_exact_f(nb[0], nb[1], nb[2], h) : godunov(nb[0], nb[1], nb[2], h);
                float out = cur;
                if (upd < cur) {
                    out = upd;
                    local = 1;
                }
                g[idx] = out;
                prev = out;
            }
        }
        if (local) changed.store(1);
    });
    (void)sa;
    return changed.load();
}

int orc_fsm_sweep(float* g, const int* dims, float h, int axis, int dir, int threads) {
    return orc_fsm_sweep_rule(g, dims, h, axis, dir, 0, threads);
}

static long long count_far(const float* g, size_t N) {
    long long c = 0;
    for (size_t i = 0; i < N; ++i) c += (g[i] >= 1e29f) ? 1 : 0;
    return c;
}

// Whole eikonal stage [D]/[D2]/[D3] (RAST:987-1064).
//   fsm_mode 0: the reference loop -- rounds of 6 sweeps until a round changes
//               nothing, at most 8; then audit-gated extra rounds (<= 16) while
//               unreached sentinels remain; then the sign-aware clamp.
//   fsm_mode 1: reference update, rounds until nothing changes (cap max_conv_rounds).
//   fsm_mode 2: corrected update, rounds until nothing changes (cap max_conv_rounds).
// Returns the rounds run; fills extra / residual / clamped.
int orc_eikonal(float* g, const uint8_t* sign, const int* dims, float h, int fsm_mode, int max_conv_rounds,
                int threads, int* extra_rounds, long long* far_residual, long long* safe_clamped) {
    const size_t N = (size_t)dims[0] * dims[1] * dims[2];
    const float bw = (float)kBandVoxels * h;
    const int rule = (fsm_mode == 2) ? 1 : 0;
    auto round6 = [&]() {
        int ch = 0;
        ch |= orc_fsm_sweep_rule(g, dims, h, 0, +1, rule, threads);
        ch |= orc_fsm_sweep_rule(g, dims, h, 0, -1, rule, threads);
        ch |= orc_fsm_sweep_rule(g, dims, h, 1, +1, rule, threads);
        ch |= orc_fsm_sweep_rule(g, dims, h, 1, -1, rule, threads);
        ch |= orc_fsm_sweep_rule(g, dims, h, 2, +1, rule, threads);
        ch |= orc_fsm_sweep_rule(g, dims, h, 2, -1, rule, threads);
        return ch;
    };
    int rounds = 0;
    int cap = (fsm_mode == 0) ? kMaxRounds : max_conv_rounds;
    for (int r = 0; r < cap; ++r) {
        int ch = round6();
        rounds = r + 1;
        if (!ch) break;
    }
    long long resid = count_far(g, N);
    int extra = 0;
    if (fsm_mode == 0) {
        while (resid > 0 && extra < kMaxExtraRounds) {
            round6();
            ++extra;
            resid = count_far(g, N);
        }
    }
    rounds += extra;
    long long clamped = 0;
    if (resid > 0) {
        clamped = resid;
        for (size_t i = 0; i < N; ++i)
            if (g[i] >= 1e29f) g[i] = (sign[i] == 1) ? -bw : bw;
        resid = count_far(g, N);
    }
    if (extra_rounds) *extra_rounds = extra;
    if (far_residual) *far_residual = resid;
    if (safe_clamped) *safe_clamped = clamped;
    return rounds;
}

// FP64 fixed point of the corrected update, from an FP32 band field (the FP64
// oracle of the exact mode). Lockstep sweeps until nothing changes; the fixed
// point of a monotone update does not depend on the schedule.
int orc_eikonal_exact_f64(const float* band, const int* dims, double h, double* out, int max_rounds, int threads) {
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    const size_t N = (size_t)dx * dy * dz;
    for (size_t i = 0; i < N; ++i) out[i] = (double)band[i];
    const long long st[3] = {1, dx, (long long)dx * dy};
    const int n[3] = {dx, dy, dz};
    std::vector<double> snap(N);
    int rounds = 0;
    for (int r = 0; r < max_rounds; ++r) {
        int ch_round = 0;
        for (int axis = 0; axis < 3; ++axis)
            for (int dir = 1; dir >= -1; dir -= 2) {
                std::memcpy(snap.data(), out, N * sizeof(double));
                int a1 = (axis == 0) ? 1 : 0, a2 = (axis == 2) ? 1 : 2;
                std::atomic<int> changed(0);
                parallel_dyn((long long)n[a1] * n[a2], 64, threads, [&](long long b, long long e) {
                    int local = 0;
                    for (long long li = b; li < e; ++li) {
                        int c[3];
                        c[a1] = (int)(li % n[a1]);
                        c[a2] = (int)(li / n[a1]);
                        double prev = 1e30;
                        for (int s = 0; s < n[axis]; ++s) {
                            c[axis] = (dir > 0) ? s : (n[axis] - 1 - s);
                            long long idx = c[0] * st[0] + c[1] * st[1] + (long long)c[2] * st[2];
                            double nb[3];
                            for (int k = 0; k < 3; ++k) {
                                double lo = (c[k] > 0) ? snap[idx - st[k]] : 1e30;
                                double hi = (c[k] < n[k] - 1) ? snap[idx + st[k]] : 1e30;
                                if (k == axis) {
                                    if (dir > 0) lo = (c[k] > 0) ? prev : 1e30;
                                    else hi = (c[k] < n[k] - 1) ? prev : 1e30;
                                }
                                nb[k] = std::min(lo, hi);
                            }
                            double upd = godunov_exact_d(nb[0], nb[1], nb[2], h);
                            double cur = snap[idx];
                            double o = cur;
                            if (upd < cur) {
                                o = upd;
                                local = 1;
                            }
                            out[idx] = o;
                            prev = o;
                        }
                    }
                    if (local) changed.store(1);
                });
                ch_round |= changed.load();
            }
        rounds = r + 1;
        if (!ch_round) break;
    }
    return rounds;
}

float orc_godunov_exact(float ax, float ay, float az, float h) { return godunov_exact_f(ax, ay, az, h); }

// ---- [E] stratified verify + patch (RAST:566-646, RAST:1078-1132) --------------------
// Undecided voxels (2) become 3, "the winding number decides", without the sum; returns
// their count, the count the fixup would return.
static long long mark_lazy(uint8_t* sign, size_t N) {
    long long n = 0;
    for (size_t i = 0; i < N; ++i)
        if (sign[i] == 2) {
            sign[i] = 3;
            ++n;
        }
    return n;
}

// Returns 1 when a probe came back clean, 0 on systematic divergence. ``lazy``: patch boxes
// are marked 3 (decided by the winding number, not summed here) and counted as patched;
// probes skip them, since the fixup and the probe make the same winding decision there.
static int verify_patch_impl(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                             const float* dist, int gwn_mode, int threads, orc_fast_stats* st, float tol, int lazy) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    const long long dx = dims[0], dy = dims[1], dz = dims[2];
    const size_t N = (size_t)(dx * dy * dz);
    for (int gen = 0; gen < kProbeGens; ++gen) {
        double off = (gen == 0) ? 0.5 : (gen == 1) ? (1.0 / 6.0) : (5.0 / 6.0);
        std::vector<long long> vidx(kVerifySamples);
        std::vector<uint8_t> ok(kVerifySamples, 1);
        for (int i = 0; i < kVerifySamples; ++i) {
            size_t v = (size_t)(((double)i + off) * (double)N / (double)kVerifySamples);
            if (v >= N) v = N - 1;
            vidx[i] = (long long)v;
        }
        GwnCounters ctr;
        parallel_dyn(kVerifySamples, 4, threads, [&](long long b, long long e) {
            for (long long i = b; i < e; ++i) {
                long long v = vidx[(size_t)i];
                uint8_t s = sign[v];
                if (s == 2 || s == 3) continue;
                int x = (int)(v % dx), y = (int)((v / dx) % dy), z = (int)(v / (dx * dy));
                V3 p{(float)(mn[0] + x) * h, (float)(mn[1] + y) * h, (float)(mn[2] + z) * h};
                bool inside = gwn_inside(tris, T, p, gwn_mode, &ctr, dist ? dist[v] : 1e30f, h, tol);
                if ((s == 1) != inside) ok[(size_t)i] = 0;
            }
        });
        st->fp64_rechecks += ctr.fp64_rechecks.load();
        std::vector<long long> sites;
        for (int i = 0; i < kVerifySamples; ++i)
            if (!ok[i]) sites.push_back(vidx[i]);
        int m = (int)sites.size();
        st->probes += 1;
        if (m == 0) return 1;
        if (m > kMaxSitesPerProbe) return 0;
        if (gen == kProbeGens - 1) return 0;
        // mark (2r+1)^3 boxes unknown (RAST:615-646) then exact fixup (RAST:1113-1116)
        for (long long v : sites) {
            int cx = (int)(v % dx), cy = (int)((v / dx) % dy), cz = (int)(v / (dx * dy));
            int x0 = std::max(0, cx - kPatchRadius), y0 = std::max(0, cy - kPatchRadius),
                z0 = std::max(0, cz - kPatchRadius);
            int x1 = std::min((int)dx - 1, cx + kPatchRadius), y1 = std::min((int)dy - 1, cy + kPatchRadius),
                z1 = std::min((int)dz - 1, cz + kPatchRadius);
            for (int z = z0; z <= z1; ++z)
                for (int y = y0; y <= y1; ++y)
                    for (int x = x0; x <= x1; ++x) sign[(size_t)z * dx * dy + (size_t)y * dx + x] = 2;
        }
        long long fixed = lazy ? mark_lazy(sign, N)
                               : orc_fixup_unknown_tol(tris_, T, h, mn, dims, sign, dist, gwn_mode, threads,
                                                       &st->fp64_rechecks, tol);
        st->patched_voxels += fixed;
        st->sites += m;
        st->patch_rounds += 1;
    }
    return 0;
}

int orc_verify_patch(const void* tris_, int T, float h, const int* mn, const int* dims, uint8_t* sign,
                     const float* dist, int gwn_mode, int threads, orc_fast_stats* st, float tol) {
    return verify_patch_impl(tris_, T, h, mn, dims, sign, dist, gwn_mode, threads, st, tol, 0);
}

// ---- [F] sign apply (RAST:650-661) --------------------------------------------------
void orc_apply_signs(float* g, const uint8_t* sign, long long N) {
    for (long long i = 0; i < N; ++i) {
        float d = g[i];
        if (d > 1e29f) d = 1e6f;
        g[i] = (sign[i] == 1) ? -d : d;
    }
}

// ---- the whole fast path (RAST:796-1159) ---------------------------------------------
// out_dist: N floats (left untouched on failure); out_sign: N bytes scratch (0/1 final; 3 marks
// a voxel left to the winding number under lazy_winding, written with a positive distance).
int orc_fast_sdf(const void* tris_, int T, float h, const int* mn, const int* mx, const orc_fast_params* prm,
                 float* out_dist, uint8_t* out_sign, orc_fast_stats* st) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    std::memset(st, 0, sizeof(*st));
    auto t0 = clk::now();
    int dims[3] = {mx[0] - mn[0] + 1, mx[1] - mn[1] + 1, mx[2] - mn[2] + 1};
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || T <= 0) return st->status = 1;
    long long N = (long long)dims[0] * dims[1] * dims[2];
    // the reference's 32-bit index guard (RAST:816-820); the exact-signs modes index in 64 bits
    if (!prm->signed_parity &&
        (N > 2000000000LL || (long long)T * dims[2] > 2000000000LL || (long long)dims[0] * dims[1] > 2000000000LL ||
         (long long)dims[0] * dims[2] > 2000000000LL || (long long)dims[1] * dims[2] > 2000000000LL))
        return st->status = 2;
    int threads = std::max(1, prm->threads);
    std::vector<float> g((size_t)N);
    // [B] needs the CSR guard before anything is written (RAST:867-869)
    auto ta = clk::now();
    st->band_voxels = orc_splat_band(tris_, T, h, mn, dims, g.data(), threads);
    auto tb = clk::now();
    long long unk = orc_parity_signs_mode(tris_, T, h, mn, dims, out_sign, threads, prm->signed_parity);
    const float tol = prm->signed_parity ? kSurfaceTolExact : kSurfaceTolVoxels;
    auto tc = clk::now();
    if (unk < 0) return st->status = 3;
    st->unknown_columns = (int)unk;
    if (unk > 0)
        st->fixup_voxels = prm->lazy_winding ? mark_lazy(out_sign, (size_t)N)
                                             : orc_fixup_unknown_tol(tris_, T, h, mn, dims, out_sign, g.data(),
                                                                     prm->gwn_mode, threads, &st->fp64_rechecks, tol);
    auto td = clk::now();
    // [D] changes no voxel at or below the surface tolerance (a Godunov update of non-negative
    // neighbours is at least h/sqrt(3)), so [E] decides the same without it.
    if (!prm->skip_eikonal)
        st->eikonal_rounds = orc_eikonal(g.data(), out_sign, dims, h, prm->fsm_mode,
                                         prm->max_conv_rounds > 0 ? prm->max_conv_rounds : 100000, threads,
                                         &st->extra_rounds, &st->far_residual, &st->safe_clamped);
    auto te = clk::now();
    int ok = prm->skip_verify ? 1
                              : verify_patch_impl(tris_, T, h, mn, dims, out_sign, g.data(), prm->gwn_mode, threads, st,
                                                  tol, prm->lazy_winding);
    auto tf = clk::now();
    st->ms_splat = ms(ta, tb);
    st->ms_parity = ms(tb, tc);
    st->ms_fixup = ms(tc, td);
    st->ms_eikonal = ms(td, te);
    st->ms_verify = ms(te, tf);
    if (!ok) {
        st->ms_total = ms(t0, clk::now());
        return st->status = 4;
    }
    if (prm->signed_parity) {  // on-surface voxels take the exact-arithmetic sign (inside)
        for (long long i = 0; i < N; ++i)
            if (g[(size_t)i] <= tol * h) out_sign[i] = 1;
    }
    orc_apply_signs(g.data(), out_sign, N);
    std::memcpy(out_dist, g.data(), (size_t)N * sizeof(float));
    auto tg = clk::now();
    st->ms_apply = ms(tf, tg);
    st->ms_total = ms(t0, tg);
    return st->status = 0;
}

// ---- legacy exact kernel (RAST:97-185; tile headers RAST:1197-1235) ------------------
void orc_legacy_sdf(const void* tris_, int T, float h, const int* mn, const int* mx, int gwn_mode, float* out,
                    int threads) {
    const OTri* tris = static_cast<const OTri*>(tris_);
    const int TILE = 128;  // RASTER_TILE_SIZE, MATH:35
    int dims[3] = {mx[0] - mn[0] + 1, mx[1] - mn[1] + 1, mx[2] - mn[2] + 1};
    const long long dx = dims[0], dy = dims[1], dz = dims[2];
    int ntiles = (T + TILE - 1) / TILE;
    std::vector<float> hb((size_t)ntiles * 6);
    for (int t = 0; t < ntiles; ++t) {
        float bmin[3] = {1e30f, 1e30f, 1e30f}, bmax[3] = {-1e30f, -1e30f, -1e30f};
        for (int i = t * TILE; i < std::min(T, (t + 1) * TILE); ++i) {
            const OTri& tr = tris[i];
            const float* vs[3] = {&tr.v0.x, &tr.v1.x, &tr.v2.x};
            for (int k = 0; k < 3; ++k) {
                // glm::min(bmin, glm::min(v0, glm::min(v1, v2)))
                float lo = std::min(vs[0][k], std::min(vs[1][k], vs[2][k]));
                float hi = std::max(vs[0][k], std::max(vs[1][k], vs[2][k]));
                bmin[k] = std::min(bmin[k], lo);
                bmax[k] = std::max(bmax[k], hi);
            }
        }
        for (int k = 0; k < 3; ++k) {
            hb[(size_t)t * 6 + k] = bmin[k];
            hb[(size_t)t * 6 + 3 + k] = bmax[k];
        }
    }
    parallel_dyn(dx * dy * dz, 64, threads, [&](long long b, long long e) {
        for (long long i = b; i < e; ++i) {
            int x = (int)(i % dx), y = (int)((i / dx) % dy), z = (int)(i / (dx * dy));
            V3 p{(float)(mn[0] + x) * h, (float)(mn[1] + y) * h, (float)(mn[2] + z) * h};
            float mind = 1e12f;
            for (int t = 0; t < ntiles; ++t) {
                const float* hh = &hb[(size_t)t * 6];
                float bdx = (p.x < hh[0]) ? (hh[0] - p.x) : ((p.x > hh[3]) ? (p.x - hh[3]) : 0.0f);
                float bdy = (p.y < hh[1]) ? (hh[1] - p.y) : ((p.y > hh[4]) ? (p.y - hh[4]) : 0.0f);
                float bdz = (p.z < hh[2]) ? (hh[2] - p.z) : ((p.z > hh[5]) ? (p.z - hh[5]) : 0.0f);
                float box = bdx * bdx + bdy * bdy + bdz * bdz;
                if (!(box < mind)) continue;
                for (int k = t * TILE; k < std::min(T, (t + 1) * TILE); ++k) {
                    float d2 = ptd_sq(p, tris[k].v0, tris[k].v1, tris[k].v2);
                    if (d2 < mind) mind = d2;
                }
            }
            bool inside = gwn_inside(tris, T, p, gwn_mode, nullptr, std::sqrt(mind), h);
            float sgn = inside ? -1.0f : 1.0f;
            out[i] = sgn * std::sqrt(mind);
        }
    });
}

// ---- build_from_mesh front-end (RAST:1340-1435; MATH:484-514) -------------------------
// Lattice: bbox over all vertices, pad 10h, floor/ceil. Returns 0 on success.
int orc_lattice(const float* verts, long long nv, float h, int* mn, int* mx) {
    if (nv <= 0) return 1;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (long long i = 0; i < nv; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::fmin(lo[k], verts[3 * i + k]);
            hi[k] = std::fmax(hi[k], verts[3 * i + k]);
        }
    float pad = h * 10.0f;
    for (int k = 0; k < 3; ++k) {
        mn[k] = (int)std::floor((lo[k] - pad) / h);
        mx[k] = (int)std::ceil((hi[k] + pad) / h);
    }
    return 0;
}

// Triangles in index order; degenerate (|cross|^2 <= 1e-12) and out-of-range faces
// dropped. Returns the kept count. (The reference compacts with atomicAdd, so its
// order is nondeterministic, RAST:1321-1337; index order is the deterministic one.)
long long orc_build_triangles(const float* verts, long long nv, const uint32_t* idx, long long nt, void* out_) {
    OTri* out = static_cast<OTri*>(out_);
    long long k = 0;
    for (long long t = 0; t < nt; ++t) {
        uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        if (i0 >= (uint64_t)nv || i1 >= (uint64_t)nv || i2 >= (uint64_t)nv) continue;
        V3 v0{verts[3 * i0], verts[3 * i0 + 1], verts[3 * i0 + 2]};
        V3 v1{verts[3 * i1], verts[3 * i1 + 1], verts[3 * i1 + 2]};
        V3 v2{verts[3 * i2], verts[3 * i2 + 1], verts[3 * i2 + 2]};
        V3 a = sub(v1, v0), b = sub(v2, v0);
        V3 n{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
        float len2 = dot(n, n);
        if (len2 > 1e-12f) {
            float inv = 1.0f / std::sqrt(len2);
            out[k].v0 = v0;
            out[k].v1 = v1;
            out[k].v2 = v2;
            out[k].n = mul(n, inv);
            ++k;
        }
    }
    return k;
}

// Reference gate for compute_mesh_sdf (RAST:1189).
long long orc_fast_min_voxels() { return (long long)kFastMinVoxels; }

}  // extern "C"
