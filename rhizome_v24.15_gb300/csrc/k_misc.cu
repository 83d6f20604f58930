// k_misc.cu — front-end and legacy-path kernels of the mesh-to-SDF engine:
//   * deterministic triangle build from an indexed mesh (build_from_mesh front-end),
//   * the legacy exact kernel's distance pass (mesh_to_sdf_kernel),
//   * small packing / combine helpers.
#include <algorithm>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

// dev_try_build_cuda_triangle (math_utils.cuh:484-514): indices in range and
// |cross(v1-v0, v2-v0)|^2 > 1e-12.
__device__ __forceinline__ bool build_one(const float* __restrict__ verts, long long nv,
                                          const uint32_t* __restrict__ idx, long long t, float* out12) {
    uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
    if ((long long)i0 >= nv || (long long)i1 >= nv || (long long)i2 >= nv) return false;
    f3 v0 = mk(verts[3ll * i0], verts[3ll * i0 + 1], verts[3ll * i0 + 2]);
    f3 v1 = mk(verts[3ll * i1], verts[3ll * i1 + 1], verts[3ll * i1 + 2]);
    f3 v2 = mk(verts[3ll * i2], verts[3ll * i2 + 1], verts[3ll * i2 + 2]);
    f3 a = sub(v1, v0), b = sub(v2, v0);
    f3 n = mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
    float len2 = dot(n, n);
    if (!(len2 > 1e-12f)) return false;
    if (out12) {
        float inv = rsqrtf(len2);
        out12[0] = v0.x; out12[1] = v0.y; out12[2] = v0.z;
        out12[3] = v1.x; out12[4] = v1.y; out12[5] = v1.z;
        out12[6] = v2.x; out12[7] = v2.y; out12[8] = v2.z;
        out12[9] = n.x * inv; out12[10] = n.y * inv; out12[11] = n.z * inv;
    }
    return true;
}

__global__ void tri_flags_kernel(const float* __restrict__ verts, long long nv, const uint32_t* __restrict__ idx,
                                 long long nt, unsigned* __restrict__ flags) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nt) flags[t] = build_one(verts, nv, idx, t, nullptr) ? 1u : 0u;
}

// Scatter kept faces to their prefix-sum slot: index order is preserved (the
// reference's atomicAdd compaction, cuda_rasterizer.cu:1321-1337, is not).
__global__ void tri_scatter_kernel(const float* __restrict__ verts, long long nv, const uint32_t* __restrict__ idx,
                                   long long nt, const unsigned long long* __restrict__ pos,
                                   float* __restrict__ out) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    float r[12];
    if (build_one(verts, nv, idx, t, r)) {
        float* o = out + 12 * pos[t];
        for (int k = 0; k < 12; ++k) o[k] = r[k];
    }
}

__global__ void pack_tri9_kernel(const float* __restrict__ t12, long long T, float* __restrict__ t9) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    for (int k = 0; k < 9; ++k) t9[9 * t + k] = t12[12 * t + k];
}

// Legacy tile headers: per 128-triangle tile the min / max of its vertices
// (cuda_rasterizer.cu:1200-1213; only the bounds are used by the active branch).
__global__ void tile_bounds_kernel(const float* __restrict__ t12, long long T, int tile, float* __restrict__ hb) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long ntiles = (T + tile - 1) / tile;
    if (k >= ntiles) return;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (long long i = k * tile; i < min(T, (k + 1) * tile); ++i)
        for (int a = 0; a < 3; ++a) {
            float v0 = t12[12 * i + a], v1 = t12[12 * i + 3 + a], v2 = t12[12 * i + 6 + a];
            lo[a] = fminf(lo[a], fminf(v0, fminf(v1, v2)));
            hi[a] = fmaxf(hi[a], fmaxf(v0, fmaxf(v1, v2)));
        }
    for (int a = 0; a < 3; ++a) {
        hb[6 * k + a] = lo[a];
        hb[6 * k + 3 + a] = hi[a];
    }
}

constexpr int kLegTile = 128;  // RASTER_TILE_SIZE (math_utils.cuh:35)

// Legacy distance pass (cuda_rasterizer.cu:97-185): per voxel, exact squared
// distance minimised over 128-triangle tiles, a tile skipped when its box distance
// is not below the running minimum (the reference's can_contain_closer test).
// Writes min d^2; the winding sign comes from the exact winding kernels.
__global__ void __launch_bounds__(256) legacy_dist_kernel(const float* __restrict__ t9, long long T,
                                                          const float* __restrict__ hb, Lattice L,
                                                          float* __restrict__ d2out) {
    __shared__ float s[kLegTile * 9];
    const long long ntiles = (T + kLegTile - 1) / kLegTile;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = v < L.N;
    int x = 0, y = 0, z = 0;
    if (ok) {
        x = (int)(v % L.dims[0]);
        long long r = v / L.dims[0];
        y = (int)(r % L.dims[1]);
        z = (int)(r / L.dims[1]);
    }
    const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
    float mind = 1e12f;
    for (long long t = 0; t < ntiles; ++t) {
        const long long t0 = t * kLegTile;
        const int m = (int)min((long long)kLegTile, T - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < m * 9; k += blockDim.x) s[k] = t9[t0 * 9 + k];
        __syncthreads();
        if (!ok) continue;
        const float* hh = hb + 6 * t;
        float bdx = (p.x < hh[0]) ? (hh[0] - p.x) : ((p.x > hh[3]) ? (p.x - hh[3]) : 0.0f);
        float bdy = (p.y < hh[1]) ? (hh[1] - p.y) : ((p.y > hh[4]) ? (p.y - hh[4]) : 0.0f);
        float bdz = (p.z < hh[2]) ? (hh[2] - p.z) : ((p.z > hh[5]) ? (p.z - hh[5]) : 0.0f);
        float box = bdx * bdx + bdy * bdy + bdz * bdz;
        if (!(box < mind)) continue;
        for (int i = 0; i < m; ++i) {
            const float* q = s + 9 * i;
            float d2 = ptd_sq(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
            if (d2 < mind) mind = d2;
        }
    }
    if (ok) d2out[v] = mind;
}

// out = (inside ? -1 : 1) * sqrt(min d^2)  (cuda_rasterizer.cu:181-184)
__global__ void legacy_combine_kernel(const float* __restrict__ d2, const uint32_t* __restrict__ sbits, Lattice L,
                                      float* __restrict__ out) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.N; i += stride) {
        long long row = i / L.dims[0];
        int x = (int)(i - row * L.dims[0]);
        bool in = (sbits[(size_t)row * L.wx + (x >> 5)] >> (x & 31)) & 1u;
        float sg = in ? -1.0f : 1.0f;
        out[i] = sg * sqrtf(d2[i]);
    }
}

// Self-test: div3_rn against the IEEE quotient x / 3.0f for every non-NaN float,
// div3_pos for every finite non-negative one, and the square roots nsqrt2_rn (packed) and
// nsqrt_rn against sqrtf on their range -- +0 and -0 and every float in [2^-100, 2^100]
// (the updates' operands at voxel sizes with pair_sqrt_ok).
__global__ void selftest_div3_kernel(unsigned long long* __restrict__ mism) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long bad = 0;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < (1ull << 32);
         i += stride) {
        const float x = __uint_as_float((unsigned)i);
        if (isnan(x)) continue;
        const float a = div3_rn(x), b = x / 3.0f;
        bad += (__float_as_uint(a) != __float_as_uint(b)) ? 1ull : 0ull;
        if (i < 0x7f800000ull) {
            bad += (__float_as_uint(div3_pos(x)) != __float_as_uint(b)) ? 1ull : 0ull;
            if (i == 0 || (i >= 0x0d800000ull && i <= 0x71800000ull)) {
                // lane 1 takes +0 at x = 0; the sign of a zero root is left open (the updates
                // subtract it from a non-negative sum, where +0 and -0 give the same value)
                float r0, r1;
                up2(nsqrt2_rn(pk2(-x, i == 0 ? 0.0f : -x), pk2(0.5f, 0.5f)), r0, r1);
                const unsigned want = __float_as_uint(-sqrtf(x)), mask = (i == 0) ? 0x7fffffffu : 0xffffffffu;
                bad += ((__float_as_uint(r0) & mask) != (want & mask)) ? 1ull : 0ull;
                bad += ((__float_as_uint(r1) & 0x7fffffffu) != (want & 0x7fffffffu)) ? 1ull : 0ull;
                bad += ((__float_as_uint(nsqrt_rn(-x)) & mask) != (want & mask)) ? 1ull : 0ull;
            }
        }
    }
    if (bad) atomicAdd(mism, bad);
}

// Self-test of the reference update's branch-free forms: godunov_ref_nb, godunov_ref_nbp
// (one voxel, packed lanes) and both lanes of godunov_ref_pair against godunov_ref (the
// reference's branches, sqrtf, div3_rn) on 2^30 generated neighbour triples. Eight voxel
// sizes across the range of pair_sqrt_ok; neighbours a random base up to 600 h plus up to
// 2 h each, with ties, exact 1D / 2D boundaries (s1 = s0 + h), far sentinels and zeros
// mixed in, so every branch of the reference rule is taken.
__device__ __forceinline__ uint32_t st_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ void st_triple(uint32_t i, float h, float* v) {
    const uint32_t r1 = st_mix(i * 4u + 1u), r2 = st_mix(i * 4u + 2u), r3 = st_mix(i * 4u + 3u);
    const float base = h * 600.0f * (float)(r1 >> 8) * 0x1p-24f;
    v[0] = base + h * 2.0f * (float)(r2 & 0xffffu) * 0x1p-16f;
    v[1] = base + h * 2.0f * (float)(r2 >> 16) * 0x1p-16f;
    v[2] = base + h * 2.0f * (float)(r3 & 0xffffu) * 0x1p-16f;
    const uint32_t k = (r3 >> 16) & 15u, a = (r3 >> 20) % 3u, b = (a + 1u + ((r3 >> 22) & 1u)) % 3u;
    if (k == 0) v[a] = kFarSentinel;
    else if (k == 1) v[a] = v[b];
    else if (k == 2) v[a] = v[b] = v[3 - a - b];
    else if (k == 3) v[a] = v[b] + h;
    else if (k == 4) v[a] = 0.0f;
    else if (k == 5) v[a] = v[b] = kFarSentinel;
}
__global__ void selftest_godunov_kernel(unsigned long long* __restrict__ mism) {
    const float hs[8] = {0.1f, 1.0f, 0.37f, 0x1p-20f, 0x1p20f, 3.3e-3f, 25.0f, 0.0625f};
    const uint32_t stride = gridDim.x * blockDim.x;
    unsigned long long bad = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (1u << 30); i += stride) {
        const float h = hs[st_mix(i ^ 0x5bd1e995u) & 7u];
        float a[3], b[3];
        st_triple(i, h, a);
        st_triple(i ^ 0x2545f491u, h, b);
        const float ra = godunov_ref(a[0], a[1], a[2], h), rb = godunov_ref(b[0], b[1], b[2], h);
        const float nb = godunov_ref_nb(a[0], a[1], a[2], h, -2.0f * h, -(3.0f * h * h));
        const float nbp = godunov_ref_nbp(a[0], a[1], a[2], godunov_one_consts(h));
        float p0, p1;
        godunov_ref_pair(a[0], a[1], a[2], b[0], b[1], b[2], godunov_pair_consts(h), p0, p1);
        const unsigned w = __float_as_uint(ra);
        bad += (__float_as_uint(nb) != w) + (__float_as_uint(nbp) != w) + (__float_as_uint(p0) != w) +
               (__float_as_uint(p1) != __float_as_uint(rb));
    }
    if (bad) atomicAdd(mism, bad);
}

__global__ void iota_kernel(long long* __restrict__ list, long long n, long long from) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) list[i] = from + i;
}

}  // namespace

void launch_pack_tri9(const float* tris12, long long T, float* tri9, cudaStream_t st) {
    if (T <= 0) return;
    GBSDF_COUNT_LAUNCH();
    pack_tri9_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(tris12, T, tri9);
}

void launch_tri_flags(const float* verts, long long nv, const uint32_t* idx, long long nt, unsigned* flags,
                      cudaStream_t st) {
    if (nt <= 0) return;
    GBSDF_COUNT_LAUNCH();
    tri_flags_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(verts, nv, idx, nt, flags);
}

void launch_tri_scatter(const float* verts, long long nv, const uint32_t* idx, long long nt,
                        const unsigned long long* pos, float* out, cudaStream_t st) {
    if (nt <= 0) return;
    GBSDF_COUNT_LAUNCH();
    tri_scatter_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(verts, nv, idx, nt, pos, out);
}

void launch_tile_bounds(const float* t12, long long T, float* hb, cudaStream_t st) {
    long long ntiles = (T + kLegTile - 1) / kLegTile;
    GBSDF_COUNT_LAUNCH();
    tile_bounds_kernel<<<(unsigned)((ntiles + 127) / 128), 128, 0, st>>>(t12, T, kLegTile, hb);
}

void launch_legacy_dist(const float* t9, long long T, const float* hb, const Lattice& L, float* d2,
                        cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    legacy_dist_kernel<<<(unsigned)((L.N + 255) / 256), 256, 0, st>>>(t9, T, hb, L, d2);
}

void launch_legacy_combine(const float* d2, const uint32_t* sbits, const Lattice& L, float* out, cudaStream_t st) {
    long long blocks = std::min<long long>((L.N + 255) / 256, 152LL * 32);
    GBSDF_COUNT_LAUNCH();
    legacy_combine_kernel<<<(unsigned)blocks, 256, 0, st>>>(d2, sbits, L, out);
}

void launch_selftest_div3(unsigned long long* mism, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    selftest_div3_kernel<<<152 * 16, 256, 0, st>>>(mism);
}

void launch_selftest_godunov(unsigned long long* mism, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    selftest_godunov_kernel<<<152 * 16, 256, 0, st>>>(mism);
}

void launch_iota(long long* list, long long n, long long from, cudaStream_t st) {
    if (n <= 0) return;
    GBSDF_COUNT_LAUNCH();
    iota_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(list, n, from);
}

namespace {
__global__ void batch_finalize_kernel(DevState* ds, int csr_guard) {
    const bool csr_bad = csr_guard && (ds->csr_entries == 0ull || ds->csr_entries > 100000000ull);
    if (ds->invalid_tris > 0ull || csr_bad || ds->overflow) ds->abort_ = 1;
}
}  // namespace

void launch_batch_finalize(DevState* ds, int csr_guard, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    batch_finalize_kernel<<<1, 1, 0, st>>>(ds, csr_guard);
}

}  // namespace gbsdf
