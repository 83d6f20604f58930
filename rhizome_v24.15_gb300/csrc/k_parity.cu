// k_parity.cu — scanline parity signs [B] with warp ballots.
//
// The reference runs one thread per (x, y) column, gathers up to 128 z-crossings
// of the jittered column ray from a host-built 4x4-supercell CSR, sorts them and
// writes one byte per voxel with column-strided stores (cuda_rasterizer.cu:279-368,
// CSR :824-882). Here one warp owns a strip of 32 adjacent columns of one row: the
// strip's candidate list is filtered 32 entries at a time by the part of the test the
// lanes share (the row), the survivors are walked uniformly by the warp, each lane keeps its own
// crossings in shared memory, and the inside/outside state of the 32 lanes at each
// z is packed into one 32-bit sign word with __ballot_sync -- one store per warp
// per z, bit-packed signs (1 bit per voxel) instead of bytes.
//
// Candidate predicate per (column, triangle), identical to the reference: the
// column's supercell lies in the triangle's CSR supercell range and the jittered
// ray passes the triangle's XY AABB; then the 2D edge functions, the |area2| >=
// 1e-12 test and the barycentric hit height. An odd or overflowing (> 128) hit
// count marks the whole column unknown (exact winding later).
#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

constexpr int kParWarps = 4;
// Exact-signs rays sit 1000x closer to the lattice point than the reference's jitter.
constexpr float kJXExact = 3.7e-4f;
constexpr float kJYExact = 5.1e-4f;

// SIGNED = 0: the reference's parity. SIGNED = 1: signed crossings -- a crossing whose
// projected triangle is clockwise in xy (entering an outward-oriented solid going up)
// counts +1, a counter-clockwise one -1; the running sum below a voxel is the winding
// number of a closed, consistently oriented mesh (overlapping shells included), inside
// iff nonzero; a column whose total is nonzero (a ray through a hole) or that overflows
// is unknown.
template <int SIGNED>
__global__ void __launch_bounds__(kParWarps * 32) parity_kernel(const ParTri* __restrict__ ptt,
                                                                const unsigned long long* __restrict__ off,
                                                                const unsigned* __restrict__ cnt,
                                                                const unsigned* __restrict__ list, Lattice L,
                                                                uint32_t* __restrict__ sbits,
                                                                uint32_t* __restrict__ ubits, DevState* ds) {
    extern __shared__ float s_hits[];  // [kParWarps][kParityMaxHits][32] floats, then signs
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long strip = (long long)blockIdx.x * kParWarps + warp;
    if (strip >= L.nstrips || ds->overflow) return;  // whole warp leaves; no block barrier below
    float* hits = s_hits + (size_t)warp * kParityMaxHits * 32;
    signed char* hsg = reinterpret_cast<signed char*>(s_hits + (size_t)kParWarps * kParityMaxHits * 32) +
                       (size_t)warp * kParityMaxHits * 32;
    const int y = (int)(strip / L.nsx), sx = (int)(strip % L.nsx);
    const int x = sx * kStrip + lane;
    const bool col = x < L.dims[0];
    const float h = L.h;
    const float rx = ((float)(L.mn[0] + x) + (SIGNED ? kJXExact : kJX)) * h;
    const float ry = ((float)(L.mn[1] + y) + (SIGNED ? kJYExact : kJY)) * h;
    const int supx = x >> 2, supy = y >> 2;
    int nh = 0;
    bool bad = false;
    const unsigned long long o = off[strip];
    const unsigned n = cnt[strip];
    for (unsigned e0 = 0; e0 < n; e0 += 32) {
        // The row part of the candidate test is the same for the 32 lanes (one row y): each
        // lane tests one list entry, and the warp walks only the entries that pass, in list
        // order. The test is the negated skip condition, so a NaN bound passes as before.
        unsigned tri = 0;
        bool row = false;
        if (e0 + lane < n) {
            tri = list[o + e0 + lane];
            const int4 sr = *reinterpret_cast<const int4*>(&ptt[tri].sx0);
            const float4 ab = *reinterpret_cast<const float4*>(ptt[tri].xyab);
            row = !(supy < sr.z || supy > sr.w || ry < ab.y || ry > ab.w);
        }
        unsigned rows = __ballot_sync(0xffffffffu, row);
        while (rows) {
            const int src = __ffs(rows) - 1;
            rows &= rows - 1;
            const ParTri& p = ptt[__shfl_sync(0xffffffffu, tri, src)];
            if (!col || bad) continue;
            if (supx < p.sx0 || supx > p.sx1) continue;
            const float4 ab = *reinterpret_cast<const float4*>(p.xyab);
            if (rx < ab.x || rx > ab.z) continue;
            const float* v = p.v;
            // the roundings of the reference's build (nvcc's default FMA contraction):
            // a*b - c*d as fma(a, b, -(c*d)), the hit height's sum as
            // fma(d0, z2, fma(d1, z0, d2*z1))
            float d0 = __fmaf_rn(v[3] - v[0], ry - v[1], -((v[4] - v[1]) * (rx - v[0])));
            float d1 = __fmaf_rn(v[6] - v[3], ry - v[4], -((v[7] - v[4]) * (rx - v[3])));
            float d2 = __fmaf_rn(v[0] - v[6], ry - v[7], -((v[1] - v[7]) * (rx - v[6])));
            bool pos = (d0 > 0.0f && d1 > 0.0f && d2 > 0.0f);
            bool neg = (d0 < 0.0f && d1 < 0.0f && d2 < 0.0f);
            if (!pos && !neg) continue;
            float area2 = d0 + d1 + d2;
            if (fabsf(area2) < 1e-12f) continue;
            float zh = __fmaf_rn(d0, v[8], __fmaf_rn(d1, v[2], d2 * v[5])) / area2;
            if (nh < kParityMaxHits) {
                hits[nh * 32 + lane] = zh;
                if (SIGNED) hsg[nh * 32 + lane] = neg ? 1 : -1;
                ++nh;
            } else {
                bad = true;
            }
        }
    }
    // insertion sort of this lane's crossings (with their signs)
    int total = 0;
    for (int i = 1; i < nh; ++i) {
        float key = hits[i * 32 + lane];
        signed char ks = SIGNED ? hsg[i * 32 + lane] : 0;
        int j = i - 1;
        while (j >= 0 && hits[j * 32 + lane] > key) {
            hits[(j + 1) * 32 + lane] = hits[j * 32 + lane];
            if (SIGNED) hsg[(j + 1) * 32 + lane] = hsg[j * 32 + lane];
            --j;
        }
        hits[(j + 1) * 32 + lane] = key;
        if (SIGNED) hsg[(j + 1) * 32 + lane] = ks;
    }
    if (SIGNED)
        for (int i = 0; i < nh; ++i) total += hsg[i * 32 + lane];
    const bool unknown = col && (bad || (SIGNED ? (total != 0) : (nh & 1)));
    const uint32_t uword = __ballot_sync(0xffffffffu, unknown);
    if (lane == 0 && uword) atomicAdd(&ds->unknown_columns, (unsigned long long)__popc(uword));
    const bool track = col && !unknown;
    int k = 0;
    bool inside = false;
    int wnum = 0;
    const size_t zrow = (size_t)L.dims[1] * L.wx;
    const size_t wbase = (size_t)y * L.wx + sx;
    for (int z = 0; z < L.dims[2]; ++z) {
        const float zc = (float)(L.mn[2] + z) * h;
        if (track) {
            while (k < nh && hits[k * 32 + lane] < zc) {
                inside = !inside;
                if (SIGNED) wnum += hsg[k * 32 + lane];
                ++k;
            }
        }
        const uint32_t sword = __ballot_sync(0xffffffffu, track && (SIGNED ? (wnum != 0) : inside));
        if (lane == 0) {
            sbits[(size_t)z * zrow + wbase] = sword;
            ubits[(size_t)z * zrow + wbase] = uword;
        }
    }
}

}  // namespace

void launch_parity(const ParTri* ptt, const unsigned long long* strip_off, const unsigned* strip_count,
                   const unsigned* strip_list, const Lattice& L, uint32_t* sbits, uint32_t* ubits, DevState* ds,
                   int signed_crossings, cudaStream_t st) {
    const int smem = kParWarps * kParityMaxHits * 32 * (int)(sizeof(float) + (signed_crossings ? 1 : 0));
    long long blocks = (L.nstrips + kParWarps - 1) / kParWarps;
    GBSDF_COUNT_LAUNCH();
    if (signed_crossings) {
        cudaFuncSetAttribute(parity_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        parity_kernel<1><<<(unsigned)blocks, kParWarps * 32, smem, st>>>(ptt, strip_off, strip_count, strip_list, L,
                                                                         sbits, ubits, ds);
    } else {
        cudaFuncSetAttribute(parity_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        parity_kernel<0><<<(unsigned)blocks, kParWarps * 32, smem, st>>>(ptt, strip_off, strip_count, strip_list, L,
                                                                         sbits, ubits, ds);
    }
}

}  // namespace gbsdf
