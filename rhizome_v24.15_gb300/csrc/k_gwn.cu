// k_gwn.cu — exact generalized-winding-number signs: the fixup [C] of unknown
// voxels and the stratified verify / patch loop [E] of the mesh-to-SDF path.
//
// Reference: gpu_exact_winding_fixup_kernel (cuda_rasterizer.cu:374-400) scans all
// N voxels and sums every triangle's solid angle for each unknown one in plain FP32
// index order; gpu_verify_sign_samples_kernel (:566-607), gpu_mark_patch_unknown_kernel
// (:615-646) and the host loop (:1078-1132) probe 3 x 4096 stratified voxels and patch
// (2*24+1)^3 boxes around mismatches.
//
// Here:
//  * unknown voxels are first compacted from the 1-bit unknown mask into a dense
//    list, so the O(voxels x triangles) kernel runs with every lane busy;
//  * the winding sum is FP32 with Kahan compensation, the triangles staged through
//    shared memory in chunks shared by the whole CTA; one voxel per thread for long
//    lists, one voxel per warp (triangles split over lanes) for short ones;
//  * every voxel whose FP32 |w| lies within 0.05 of 0.5 is re-evaluated in FP64 by a
//    CTA (deterministic tree reduction), so each inside/outside decision is the
//    exact-arithmetic one: inside iff |w| >= 0.5, the reference's rule;
//  * the probe / patch control runs on the device (state in DevState), so the loop
//    needs no host round trip per probe.
#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

constexpr int kGwnThreads = 256;
constexpr int kGwnChunk = 256;  // triangles staged per chunk (9 floats each)

__device__ __forceinline__ void voxel_coords(const Lattice& L, long long v, int& x, int& y, int& z) {
    long long dx = L.dims[0], dy = L.dims[1];
    x = (int)(v % dx);
    long long r = v / dx;
    y = (int)(r % dy);
    z = (int)(r / dy);
}

__device__ __forceinline__ size_t word_of(const Lattice& L, int x, int y, int z) {
    return ((size_t)z * L.dims[1] + y) * L.wx + (x >> 5);
}

__device__ __forceinline__ void consume(const Lattice& L, long long v, bool inside, int consumer,
                                        uint32_t* sbits, DevState* ds) {
    int x, y, z;
    voxel_coords(L, v, x, y, z);
    size_t w = word_of(L, x, y, z);
    uint32_t bit = 1u << (x & 31);
    if (consumer == kGwnFixup) {
        if (inside) atomicOr(&sbits[w], bit);
    } else {
        bool s = (sbits[w] & bit) != 0u;
        if (s != inside) {
            int m = atomicAdd(&ds->probe_m, 1);
            if (m < kVerifySamples) ds->sites[m] = v;
        }
    }
}

__global__ void list_unknown_kernel(uint32_t* __restrict__ ubits, uint32_t* __restrict__ sbits,
                                    uint32_t* __restrict__ ebits, Lattice L, long long* __restrict__ list,
                                    long long cap, DevState* ds, int only_if_patching) {
    if (only_if_patching && !ds->patching) return;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < L.nwords; w += stride) {
        uint32_t u = ubits[w];
        if (u == 0u) continue;
        int n = __popc(u);
        unsigned long long pos = atomicAdd(&ds->listed, (unsigned long long)n);
        if ((long long)(pos + n) > cap) {
            for (long long k = (long long)pos; k < cap && k < (long long)pos + n; ++k) list[k] = -1;
            atomicAdd(&ds->list_overflow, 1ull);
            continue;
        }
        long long row = w / L.wx;
        int xw = (int)(w % L.wx);
        long long base = row * L.dims[0] + (long long)xw * 32;
        uint32_t m = u;
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1u;
            list[pos++] = base + b;
        }
        ubits[w] = 0u;
        sbits[w] &= ~u;
        if (ebits) ebits[w] |= u;  // these voxels are now decided by the exact winding number
        if (only_if_patching) atomicAdd(&ds->patched_voxels, (unsigned long long)n);
        else atomicAdd(&ds->fixup_voxels, (unsigned long long)n);
    }
}

// Kahan step
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

template <int TEAM>
__global__ void __launch_bounds__(kGwnThreads) gwn_kernel(const float* __restrict__ tri9, long long T, Lattice L,
                                                          const long long* __restrict__ list, long long cap,
                                                          int consumer, int only_if, uint32_t* __restrict__ sbits,
                                                          long long* __restrict__ recheck, long long recheck_cap,
                                                          const float* __restrict__ dist, int dist_sq,
                                                          float surf_tol_vox, DevState* ds) {
    if (only_if && !ds->patching) return;
    const float tau = surf_tol_vox * L.h;
    constexpr int VPB = kGwnThreads / TEAM;
    __shared__ float s_tri[kGwnChunk * 9];
    const long long n = min((long long)ds->listed, cap);
    const int member = threadIdx.x % TEAM;
    const int slot = threadIdx.x / TEAM;
    unsigned long long pairs = 0;
    for (long long base = (long long)blockIdx.x * VPB; base < n; base += (long long)gridDim.x * VPB) {
        const long long j = base + slot;
        long long v = (j < n) ? list[j] : -1;
        f3 p = mk(0.f, 0.f, 0.f);
        if (v >= 0) {
            int x, y, z;
            voxel_coords(L, v, x, y, z);
            p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
            if (dist) {
                const float d = dist[v];
                if (dist_sq ? (d <= tau * tau) : (d <= tau)) {  // on the surface: inside
                    if (member == 0) consume(L, v, true, consumer, sbits, ds);
                    v = -2;
                }
            }
        }
        float s = 0.0f, c = 0.0f;
        bool amb = false;
        for (long long c0 = 0; c0 < T; c0 += kGwnChunk) {
            int m = (int)min((long long)kGwnChunk, T - c0);
            __syncthreads();
            for (int k = threadIdx.x; k < m * 9; k += kGwnThreads) s_tri[k] = __ldg(tri9 + c0 * 9 + k);
            __syncthreads();
            if (v >= 0) {
                for (int i = member; i < m; i += TEAM) {
                    const float* t = s_tri + i * 9;
                    kahan_add(s, c, solid_angle_fast(p, mk(t[0], t[1], t[2]), mk(t[3], t[4], t[5]),
                                                     mk(t[6], t[7], t[8]), amb));
                }
            }
        }
        if constexpr (TEAM > 1) {
            // combine the lanes' compensated partials in a fixed order
            float tot = s - c;
#pragma unroll
            for (int o = TEAM / 2; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o, TEAM);
            s = tot;
            c = 0.0f;
            amb = __any_sync(0xffffffffu, amb);
        }
        if (v >= 0 && member == 0) {
            pairs += (unsigned long long)T;
            float w = (s - c) * kInv4Pi;
            float aw = fabsf(w);
            if (amb || fabsf(aw - 0.5f) < kRecheckBand) {
                unsigned long long r = atomicAdd(&ds->recheck_n, 1ull);
                if ((long long)r < recheck_cap) recheck[r] = v;
            } else {
                consume(L, v, aw >= 0.5f, consumer, sbits, ds);
            }
        }
    }
    if (pairs) atomicAdd(&ds->gwn_pairs, pairs);
}

// The per-triangle sum for the voxels the cluster stages leave (launch_gwn_team): as
// gwn_kernel<32>, but a short list (the usual case) cuts the triangles into S fixed slices
// (S up to 32, as many as the list buffer holds partials for, behind its n entries), one CTA
// per (8 voxels, slice); gwn_sliced_final_kernel adds each voxel's partials in slice order
// and decides, so the result does not depend on the launch.
__device__ __forceinline__ int team_slices(long long n, long long cap) {
    if (n <= 0) return 1;
    return (int)max(1LL, min(32LL, (cap - n) / n));
}

__global__ void __launch_bounds__(kGwnThreads) gwn_sliced_kernel(const float* __restrict__ tri9, long long T, Lattice L,
                                                                 long long* __restrict__ list, long long cap,
                                                                 int consumer, int only_if,
                                                                 uint32_t* __restrict__ sbits,
                                                                 long long* __restrict__ recheck,
                                                                 long long recheck_cap, const float* __restrict__ dist,
                                                                 int dist_sq, float surf_tol_vox, DevState* ds) {
    if (only_if && !ds->patching) return;
    const float tau = surf_tol_vox * L.h;
    constexpr int VPB = kGwnThreads / 32;
    __shared__ float s_tri[kGwnChunk * 9];
    const long long n = min((long long)ds->listed, cap);
    const int S = team_slices(n, cap);
    float2* partial = reinterpret_cast<float2*>(list + n);
    const int member = threadIdx.x & 31;
    const int slot = threadIdx.x >> 5;
    const long long ng = (n + VPB - 1) / VPB;
    unsigned long long pairs = 0;
    for (long long it = blockIdx.x; it < ng * S; it += gridDim.x) {
        const long long grp = it / S;
        const int sl = (int)(it - grp * S);
        const long long j = grp * VPB + slot;
        long long v = (j < n) ? list[j] : -1;
        f3 p = mk(0.f, 0.f, 0.f);
        if (v >= 0) {
            int x, y, z;
            voxel_coords(L, v, x, y, z);
            p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
            if (dist) {
                const float d = dist[v];
                if (dist_sq ? (d <= tau * tau) : (d <= tau)) {  // on the surface: inside
                    if (member == 0 && sl == 0) consume(L, v, true, consumer, sbits, ds);
                    v = -2;
                }
            }
        }
        const long long t0 = T * sl / S, t1 = T * (sl + 1) / S;
        float s = 0.0f, c = 0.0f;
        bool amb = false;
        for (long long c0 = t0; c0 < t1; c0 += kGwnChunk) {
            const int m = (int)min((long long)kGwnChunk, t1 - c0);
            __syncthreads();
            for (int k = threadIdx.x; k < m * 9; k += kGwnThreads) s_tri[k] = __ldg(tri9 + c0 * 9 + k);
            __syncthreads();
            if (v >= 0) {
                for (int i = member; i < m; i += 32) {
                    const float* t = s_tri + i * 9;
                    kahan_add(s, c, solid_angle_fast(p, mk(t[0], t[1], t[2]), mk(t[3], t[4], t[5]),
                                                     mk(t[6], t[7], t[8]), amb));
                }
            }
        }
        float tot = s - c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
        amb = __any_sync(0xffffffffu, amb);
        if (member == 0 && j < n) {
            if (S > 1) {
                partial[j * S + sl] = make_float2(tot, (v >= 0) ? (amb ? 1.0f : 0.0f) : 2.0f);
            } else if (v >= 0) {
                pairs += (unsigned long long)T;
                const float aw = fabsf(tot * kInv4Pi);
                if (amb || fabsf(aw - 0.5f) < kRecheckBand) {
                    const unsigned long long r = atomicAdd(&ds->recheck_n, 1ull);
                    if ((long long)r < recheck_cap) recheck[r] = v;
                } else {
                    consume(L, v, aw >= 0.5f, consumer, sbits, ds);
                }
            }
        }
    }
    if (pairs) atomicAdd(&ds->gwn_pairs, pairs);
}

__global__ void gwn_sliced_final_kernel(long long T, Lattice L, const long long* __restrict__ list, long long cap,
                                        int consumer, int only_if, uint32_t* __restrict__ sbits,
                                        long long* __restrict__ recheck, long long recheck_cap, DevState* ds) {
    if (only_if && !ds->patching) return;
    const long long n = min((long long)ds->listed, cap);
    const int S = team_slices(n, cap);
    if (S == 1) return;
    const float2* partial = reinterpret_cast<const float2*>(list + n);
    unsigned long long pairs = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long v = list[i];
        if (v < 0 || partial[i * S].y == 2.0f) continue;  // not listed, or decided on the surface
        float tot = 0.0f;
        bool amb = false;
        for (int k = 0; k < S; ++k) {
            const float2 q = partial[i * S + k];
            tot += q.x;
            amb |= q.y != 0.0f;
        }
        pairs += (unsigned long long)T;
        const float aw = fabsf(tot * kInv4Pi);
        if (amb || fabsf(aw - 0.5f) < kRecheckBand) {
            const unsigned long long r = atomicAdd(&ds->recheck_n, 1ull);
            if ((long long)r < recheck_cap) recheck[r] = v;
        } else {
            consume(L, v, aw >= 0.5f, consumer, sbits, ds);
        }
    }
    if (pairs) atomicAdd(&ds->gwn_pairs, pairs);
}

// ---- hierarchical winding numbers (clusters of the 8^3 brick of each centroid) --------
#ifndef GBSDF_FWN_BETA
#define GBSDF_FWN_BETA 4.0f
#endif
constexpr float kFwnBeta = GBSDF_FWN_BETA;  // a cluster is far when d > beta r
constexpr float kFwnBetaFine = 16.0f;       // the refining stage's threshold
constexpr long long kFwnFineMinTris = 1000000;  // meshes that get the refining stage
constexpr float kFwnSlackRel = 1e-5f;  // rounding slack per unit of summed |terms|
constexpr float kFwnSlackAbs = 1e-5f;  // rounding slack in w

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void fwn_count_kernel(const float* __restrict__ t9, long long T, Lattice L, FwnGrid g,
                                 unsigned* __restrict__ cell_of, unsigned* __restrict__ counts) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float* v = t9 + 9 * t;
    const float inv = 1.0f / L.h;
    int b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float gc = (v[k] + v[3 + k] + v[6 + k]) * (1.0f / 3.0f);
        const float rel = gc * inv - (float)L.mn[k];
        const float c = floorf(rel / (float)g.s);
        b[k] = clampi(c != c ? 0 : (int)fmaxf(fminf(c, 1e9f), -1e9f), 0, g.n[k] - 1);
    }
    const unsigned cell = (unsigned)(((long long)b[2] * g.n[1] + b[1]) * g.n[0] + b[0]);
    cell_of[t] = cell;
    atomicAdd(&counts[cell], 1u);
}

__global__ void fwn_flag_kernel(const unsigned* __restrict__ counts, long long nb, unsigned* __restrict__ flag) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) flag[b] = counts[b] ? 1u : 0u;
}

__global__ void fwn_fill_kernel(long long T, const unsigned* __restrict__ cell_of,
                                const unsigned long long* __restrict__ off, unsigned* __restrict__ cursor,
                                unsigned* __restrict__ tri) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const unsigned c = cell_of[t];
    tri[off[c] + atomicAdd(&cursor[c], 1u)] = (unsigned)t;
}

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// one warp per grid cell: FP64 statistics, the lanes splitting the cell's triangles;
// the radius about the stored (FP32) centroid, rounded up
__global__ void fwn_stats_kernel(const float* __restrict__ t9, long long ncg, const unsigned* __restrict__ counts,
                                 const unsigned long long* __restrict__ off, const unsigned* __restrict__ flag,
                                 const unsigned long long* __restrict__ cidx, const unsigned* __restrict__ tri,
                                 FwnCell* __restrict__ cells, DevState* ds, FwnGrid g, int snx, int sny,
                                 unsigned* __restrict__ sup_of) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= ncg) return;
    if (b == ncg - 1 && lane == 0) ds->fwn_cells = cidx[b] + flag[b];
    const unsigned n = counts[b];
    if (!n) return;
    if (lane == 0) {  // the super cube of this cluster (4^3 cluster cubes)
        const long long bx = b % g.n[0], by = (b / g.n[0]) % g.n[1], bz = b / ((long long)g.n[0] * g.n[1]);
        sup_of[cidx[b]] = (unsigned)(((bz >> 2) * sny + (by >> 2)) * snx + (bx >> 2));
    }
    const unsigned long long o = off[b];
    double A = 0.0, D[3] = {0, 0, 0}, G[3] = {0, 0, 0}, mean[3] = {0, 0, 0};
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // sum_t D_t g_t^T; shifted to c below
    for (unsigned k = lane; k < n; k += 32) {
        const float* v = t9 + 9ull * tri[o + k];
        const double e1x = (double)v[3] - v[0], e1y = (double)v[4] - v[1], e1z = (double)v[5] - v[2];
        const double e2x = (double)v[6] - v[0], e2y = (double)v[7] - v[1], e2z = (double)v[8] - v[2];
        const double Dt[3] = {0.5 * (e1y * e2z - e1z * e2y), 0.5 * (e1z * e2x - e1x * e2z),
                              0.5 * (e1x * e2y - e1y * e2x)};
        const double a = sqrt(Dt[0] * Dt[0] + Dt[1] * Dt[1] + Dt[2] * Dt[2]);
        const double gt[3] = {((double)v[0] + v[3] + v[6]) / 3.0, ((double)v[1] + v[4] + v[7]) / 3.0,
                              ((double)v[2] + v[5] + v[8]) / 3.0};
        A += a;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            D[i] += Dt[i];
            G[i] += a * gt[i];
            mean[i] += gt[i];
#pragma unroll
            for (int j2 = 0; j2 < 3; ++j2) M[3 * i + j2] += Dt[i] * gt[j2];
        }
    }
    A = warp_sum_d(A);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        D[i] = warp_sum_d(D[i]);
        G[i] = warp_sum_d(G[i]);
        mean[i] = warp_sum_d(mean[i]);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = warp_sum_d(M[i]);
    const double c0 = (A > 0.0) ? G[0] / A : mean[0] / n;
    const double c1 = (A > 0.0) ? G[1] / A : mean[1] / n;
    const double c2 = (A > 0.0) ? G[2] / A : mean[2] / n;
    const float fc[3] = {(float)c0, (float)c1, (float)c2};
    double r2 = 0.0;
    for (unsigned k = lane; k < n; k += 32) {
        const float* v = t9 + 9ull * tri[o + k];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double dx = (double)v[3 * q] - fc[0], dy = (double)v[3 * q + 1] - fc[1],
                         dz = (double)v[3 * q + 2] - fc[2];
            r2 = fmax(r2, dx * dx + dy * dy + dz * dz);
        }
    }
#pragma unroll
    for (int off2 = 16; off2 > 0; off2 >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, off2));
    if (lane != 0) return;
    FwnCell c;
    c.cx = fc[0];
    c.cy = fc[1];
    c.cz = fc[2];
    c.r = (float)(sqrt(r2) * (1.0 + 1e-6)) + 1e-30f;
    c.ax = (float)D[0];
    c.ay = (float)D[1];
    c.az = (float)D[2];
    c.area = (float)(A * (1.0 + 1e-6));
    // moment about the stored centroid: sum D_t (g_t - c)^T = M - D c^T
    for (int i = 0; i < 3; ++i)
        for (int j2 = 0; j2 < 3; ++j2) c.m[3 * i + j2] = (float)(M[3 * i + j2] - D[i] * (double)fc[j2]);
    c.off = (unsigned)o;
    c.cnt = n;
    c.pad0 = 0;
    cells[cidx[b]] = c;
}

// ---- super-clusters ---------------------------------------------------------------
__global__ void fwn_sup_count_kernel(const DevState* ds, const unsigned* __restrict__ sup_of,
                                     unsigned* __restrict__ sup_counts) {
    const long long n = (long long)ds->fwn_cells;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sup_counts[sup_of[k]], 1u);
}

__global__ void fwn_sup_fill_kernel(const DevState* ds, const unsigned* __restrict__ sup_of,
                                    const unsigned long long* __restrict__ sup_off, unsigned* __restrict__ cursor,
                                    unsigned* __restrict__ child) {
    const long long n = (long long)ds->fwn_cells;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned s = sup_of[k];
        child[sup_off[s] + atomicAdd(&cursor[s], 1u)] = (unsigned)k;
    }
}

// One warp per super cube: its children sorted ascending (the fill's order is the atomics'),
// then the aggregated moments in FP64: area A = sum A_c, area vector D = sum D_c, centroid
// C = sum A_c c_c / A, first moment about C, M = sum (M_c + D_c (c_c - C)^T) (the moments
// of the triangles themselves, shifted), radius R = max (|c_c - C| + r_c): every triangle
// point lies within R of C, so the cluster bound holds with (C, R, A).
__global__ void fwn_sup_stats_kernel(long long nsc, const unsigned* __restrict__ counts,
                                     const unsigned long long* __restrict__ off, const unsigned* __restrict__ flag,
                                     const unsigned long long* __restrict__ cidx, unsigned* __restrict__ child,
                                     const FwnCell* __restrict__ cells, FwnCell* __restrict__ supers,
                                     DevState* ds) {
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= nsc) return;
    if (b == nsc - 1 && lane == 0) ds->fwn_supers = cidx[b] + flag[b];
    const unsigned n = counts[b];
    if (!n) return;
    unsigned* ch = child + off[b];
    // n <= 64: two per lane; rank = number of smaller children
    const unsigned a0 = (lane < (int)n) ? ch[lane] : 0xffffffffu;
    const unsigned a1 = (lane + 32 < (int)n) ? ch[lane + 32] : 0xffffffffu;
    unsigned r0 = 0, r1 = 0;
    for (int i = 0; i < 64; ++i) {
        const unsigned v = __shfl_sync(0xffffffffu, i < 32 ? a0 : a1, i & 31);
        r0 += v < a0;
        r1 += v < a1;
    }
    __syncwarp();
    if (lane < (int)n) ch[r0] = a0;
    if (lane + 32 < (int)n) ch[r1] = a1;
    __syncwarp();
    double A = 0.0, D[3] = {0, 0, 0}, G[3] = {0, 0, 0}, mean[3] = {0, 0, 0};
    for (unsigned k = lane; k < n; k += 32) {
        const FwnCell c = cells[ch[k]];
        A += c.area;
        const double cc[3] = {c.cx, c.cy, c.cz}, dd[3] = {c.ax, c.ay, c.az};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            D[i] += dd[i];
            G[i] += (double)c.area * cc[i];
            mean[i] += cc[i];
        }
    }
    A = warp_sum_d(A);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        D[i] = warp_sum_d(D[i]);
        G[i] = warp_sum_d(G[i]);
        mean[i] = warp_sum_d(mean[i]);
    }
    double C[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) C[i] = (A > 0.0) ? G[i] / A : mean[i] / n;
    const float fc[3] = {(float)C[0], (float)C[1], (float)C[2]};
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, R = 0.0;
    for (unsigned k = lane; k < n; k += 32) {
        const FwnCell c = cells[ch[k]];
        const double sh[3] = {(double)c.cx - fc[0], (double)c.cy - fc[1], (double)c.cz - fc[2]};
        const double dd[3] = {c.ax, c.ay, c.az};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) M[3 * i + j] += (double)c.m[3 * i + j] + dd[i] * sh[j];
        R = fmax(R, sqrt(sh[0] * sh[0] + sh[1] * sh[1] + sh[2] * sh[2]) + (double)c.r);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = warp_sum_d(M[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) R = fmax(R, __shfl_xor_sync(0xffffffffu, R, o));
    if (lane != 0) return;
    FwnCell S;
    S.cx = fc[0];
    S.cy = fc[1];
    S.cz = fc[2];
    S.r = (float)(R * (1.0 + 1e-6)) + 1e-30f;
    S.ax = (float)D[0];
    S.ay = (float)D[1];
    S.az = (float)D[2];
    S.area = (float)(A * (1.0 + 1e-6));
    for (int i = 0; i < 9; ++i) S.m[i] = (float)M[i];
    S.off = (unsigned)off[b];
    S.cnt = n;
    S.pad0 = 0;
    supers[cidx[b]] = S;
}

// far-field term of a cluster (or super-cluster) seen from p, with its truncation bound
__device__ __forceinline__ void fwn_far(const FwnCell& cl, float dx, float dy, float dz, float d2, float d, float& s,
                                        float& c, float& mag, float& err) {
    const float inv3 = 1.0f / (d2 * d);
    const float dip = (cl.ax * dx + cl.ay * dy + cl.az * dz) * inv3;
    const float tr = cl.m[0] + cl.m[4] + cl.m[8];
    const float my0 = cl.m[0] * dx + cl.m[1] * dy + cl.m[2] * dz;
    const float my1 = cl.m[3] * dx + cl.m[4] * dy + cl.m[5] * dz;
    const float my2 = cl.m[6] * dx + cl.m[7] * dy + cl.m[8] * dz;
    const float yMy = dx * my0 + dy * my1 + dz * my2;
    const float quad = (tr - 3.0f * yMy / d2) * inv3;
    kahan_add(s, c, dip + quad);
    mag += fabsf(dip) + fabsf(quad);
    const float e = (d - cl.r) * 0.99999f;
    err += 3.0f * cl.r * cl.r * cl.area / (e * e * e * e);
}

// Per-warp lists of a voxel's near clusters: their triangles are summed with the lanes
// splitting the concatenated triangle ranges evenly (a lane per cluster would leave most
// lanes idle while one walks a long cluster).
constexpr int kNearClCap = 448;

// exclusive prefix of n counts (cnt(i) for i < n) into pre[0..n]; returns the total
template <class C>
__device__ __forceinline__ unsigned warp_prefix(int n, unsigned* pre, int lane, C cnt) {
    unsigned base = 0;
    for (int b = 0; b < n; b += 32) {
        const int i = b + lane;
        const unsigned v = (i < n) ? cnt(i) : 0u;
        unsigned inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (i < n) pre[i + 1] = base + inc;
        base += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) pre[0] = 0;
    __syncwarp();
    return base;
}

__device__ __forceinline__ void warp_near_triangles(const float* __restrict__ t9, const FwnCell* __restrict__ cells,
                                                    const unsigned* __restrict__ tri, f3 p, const unsigned* ids,
                                                    unsigned* pre, int nc, int lane, float& s, float& c, float& mag,
                                                    bool& amb) {
    const unsigned total = warp_prefix(nc, pre, lane, [&](int i) { return cells[ids[i]].cnt; });
    int i = 0;
    for (unsigned g = lane; g < total; g += 32) {
        while (pre[i + 1] <= g) ++i;
        const float* tv = t9 + 9ull * tri[cells[ids[i]].off + (g - pre[i])];
        const float term =
            solid_angle_fast(p, mk(tv[0], tv[1], tv[2]), mk(tv[3], tv[4], tv[5]), mk(tv[6], tv[7], tv[8]), amb);
        kahan_add(s, c, term);
        mag += fabsf(term);
    }
    __syncwarp();
}

// One warp per listed voxel: far clusters by their dipole with the error bound, near
// clusters triangle by triangle; lane 0 decides or hands the voxel to the exact sum.
__global__ void __launch_bounds__(kGwnThreads) fwn_query_kernel(
    const float* __restrict__ t9, const FwnCell* __restrict__ cells, const unsigned* __restrict__ tri, Lattice L,
    const long long* __restrict__ list, long long cap, int consumer, int only_if, uint32_t* __restrict__ sbits,
    const float* __restrict__ dist, int dist_sq, float surf_tol_vox, DevState* ds, long long* __restrict__ fb,
    long long fb_cap, float beta, unsigned long long* __restrict__ fb_n, int last) {
    if (only_if && !ds->patching) return;
    const float tau = surf_tol_vox * L.h;
    const long long n = min((long long)ds->listed, cap);
    const long long ncells = (long long)ds->fwn_cells;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    __shared__ unsigned cl_ids[kGwnThreads / 32][kNearClCap];
    __shared__ unsigned cl_pre[kGwnThreads / 32][kNearClCap + 1];
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long certified = 0, handed = 0;
    for (long long j = warp; j < n; j += nwarps) {
        const long long v = list[j];
        if (v < 0) continue;
        int x, y, z;
        voxel_coords(L, v, x, y, z);
        const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
        if (dist) {
            const float d = dist[v];
            if (dist_sq ? (d <= tau * tau) : (d <= tau)) {  // on the surface: inside
                if (lane == 0) consume(L, v, true, consumer, sbits, ds);
                continue;
            }
        }
        float s = 0.0f, c = 0.0f, err = 0.0f, mag = 0.0f;
        bool amb = false;
        // far clusters by their moments; near ones listed (ballot slots, cluster order)
        // and their triangles summed across the lanes
        int ncl = 0;
        for (long long base = 0; base < ncells; base += 32) {
            const long long k = base + lane;
            bool nearby = false;
            if (k < ncells) {
                const FwnCell cl = cells[k];
                const float dx = cl.cx - p.x, dy = cl.cy - p.y, dz = cl.cz - p.z;
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float d = sqrtf(d2);
                if (d > beta * cl.r) fwn_far(cl, dx, dy, dz, d2, d, s, c, mag, err);
                else nearby = true;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, nearby);
            if (nearby) {
                const int slot = ncl + __popc(bal & ((1u << lane) - 1u));
                if (slot < kNearClCap) {
                    cl_ids[wib][slot] = (unsigned)k;
                } else {  // list full: this lane sums the cluster itself
                    const FwnCell cl = cells[k];
                    for (unsigned q = 0; q < cl.cnt; ++q) {
                        const float* tv = t9 + 9ull * tri[cl.off + q];
                        const float term = solid_angle_fast(p, mk(tv[0], tv[1], tv[2]), mk(tv[3], tv[4], tv[5]),
                                                            mk(tv[6], tv[7], tv[8]), amb);
                        kahan_add(s, c, term);
                        mag += fabsf(term);
                    }
                }
            }
            ncl += __popc(bal);
        }
        __syncwarp();
        warp_near_triangles(t9, cells, tri, p, cl_ids[wib], cl_pre[wib], min(ncl, kNearClCap), lane, s, c, mag, amb);
        float tot = s - c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
            err += __shfl_xor_sync(0xffffffffu, err, o);
            mag += __shfl_xor_sync(0xffffffffu, mag, o);
        }
        amb = __any_sync(0xffffffffu, amb);
        if (lane == 0) {
            const float w = fabsf(tot * kInv4Pi);
            const float E = (err + kFwnSlackRel * mag) * kInv4Pi + kFwnSlackAbs;
            if (!amb && w - E >= 0.5f) {
                consume(L, v, true, consumer, sbits, ds);
                ++certified;
            } else if (!amb && w + E < 0.5f) {
                consume(L, v, false, consumer, sbits, ds);
                ++certified;
            } else {
                const unsigned long long k = atomicAdd(fb_n, 1ull);
                if ((long long)k < fb_cap) fb[k] = v;
                ++handed;
            }
        }
    }
    if (lane == 0) {
        if (certified) atomicAdd(&ds->fwn_certified, certified);
        if (handed && last) atomicAdd(&ds->fwn_fallback_total, handed);
    }
}

constexpr int kNearCap = 192;  // near super-clusters listed per voxel (the rest expand in-lane)

// First stage: one warp per listed voxel over the super-clusters -- far ones by their
// moments and bound, near ones cluster by cluster (far clusters by moments, near ones
// triangle by triangle); lane 0 decides or hands the voxel to the cluster stage (fb2),
// whose tighter bounds decide most of what is left.
__global__ void __launch_bounds__(kGwnThreads) fwn_query_sup_kernel(
    const float* __restrict__ t9, const FwnCell* __restrict__ cells, const unsigned* __restrict__ tri,
    const FwnCell* __restrict__ supers, const unsigned* __restrict__ child, Lattice L,
    const long long* __restrict__ list, long long cap, int consumer, int only_if, uint32_t* __restrict__ sbits,
    const float* __restrict__ dist, int dist_sq, float surf_tol_vox, DevState* ds, long long* __restrict__ fb2,
    long long fb_cap) {
    if (only_if && !ds->patching) return;
    const float tau = surf_tol_vox * L.h;
    const long long n = min((long long)ds->listed, cap);
    const long long nsup = (long long)ds->fwn_supers;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    __shared__ unsigned near_list[kGwnThreads / 32][kNearCap];
    __shared__ unsigned s_pre[kGwnThreads / 32][kNearCap + 1];
    __shared__ unsigned cl_ids[kGwnThreads / 32][kNearClCap];
    __shared__ unsigned cl_pre[kGwnThreads / 32][kNearClCap + 1];
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long certified = 0;
    for (long long j = warp; j < n; j += nwarps) {
        const long long v = list[j];
        if (v < 0) continue;
        int x, y, z;
        voxel_coords(L, v, x, y, z);
        const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
        if (dist) {
            const float d = dist[v];
            if (dist_sq ? (d <= tau * tau) : (d <= tau)) {  // on the surface: inside
                if (lane == 0) consume(L, v, true, consumer, sbits, ds);
                continue;
            }
        }
        float s = 0.0f, c = 0.0f, err = 0.0f, mag = 0.0f;
        bool amb = false;
        // a near cluster: its moments when far enough, else its triangles
        auto near_cluster = [&](const FwnCell& cl) {
            const float ex = cl.cx - p.x, ey = cl.cy - p.y, ez = cl.cz - p.z;
            const float e2 = ex * ex + ey * ey + ez * ez;
            const float e = sqrtf(e2);
            if (e > kFwnBeta * cl.r) {
                fwn_far(cl, ex, ey, ez, e2, e, s, c, mag, err);
            } else {
                for (unsigned t = 0; t < cl.cnt; ++t) {
                    const float* tv = t9 + 9ull * tri[cl.off + t];
                    const float term = solid_angle_fast(p, mk(tv[0], tv[1], tv[2]), mk(tv[3], tv[4], tv[5]),
                                                        mk(tv[6], tv[7], tv[8]), amb);
                    kahan_add(s, c, term);
                    mag += fabsf(term);
                }
            }
        };
        // far super-clusters by their moments; near ones listed (in super-cluster order,
        // slots from a ballot) and their children then split across the lanes
        int nn = 0;
        for (long long base = 0; base < nsup; base += 32) {
            const long long k = base + lane;
            bool nearby = false;
            if (k < nsup) {
                const FwnCell S = supers[k];
                const float dx = S.cx - p.x, dy = S.cy - p.y, dz = S.cz - p.z;
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float d = sqrtf(d2);
                if (d > kFwnBeta * S.r) fwn_far(S, dx, dy, dz, d2, d, s, c, mag, err);
                else nearby = true;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, nearby);
            if (nearby) {
                const int slot = nn + __popc(bal & ((1u << lane) - 1u));
                if (slot < kNearCap) {
                    near_list[wib][slot] = (unsigned)k;
                } else {  // list full: this lane expands it itself
                    const FwnCell S = supers[k];
                    for (unsigned q = 0; q < S.cnt; ++q) near_cluster(cells[child[S.off + q]]);
                }
            }
            nn += __popc(bal);
        }
        __syncwarp();
        nn = min(nn, kNearCap);
        // children of the near super-clusters, concatenated and split across the lanes: far
        // ones by their moments, near ones listed for the triangle pass
        const unsigned totalS =
            warp_prefix(nn, s_pre[wib], lane, [&](int i) { return supers[near_list[wib][i]].cnt; });
        int ncl = 0, si = 0;
        for (unsigned gb = 0; gb < totalS; gb += 32) {
            const unsigned g = gb + lane;
            bool nearby = false;
            unsigned cid = 0;
            if (g < totalS) {
                while (s_pre[wib][si + 1] <= g) ++si;
                cid = child[supers[near_list[wib][si]].off + (g - s_pre[wib][si])];
                const FwnCell cl = cells[cid];
                const float ex = cl.cx - p.x, ey = cl.cy - p.y, ez = cl.cz - p.z;
                const float e2 = ex * ex + ey * ey + ez * ez;
                const float e = sqrtf(e2);
                if (e > kFwnBeta * cl.r) fwn_far(cl, ex, ey, ez, e2, e, s, c, mag, err);
                else nearby = true;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, nearby);
            if (nearby) {
                const int slot = ncl + __popc(bal & ((1u << lane) - 1u));
                if (slot < kNearClCap) cl_ids[wib][slot] = cid;
                else near_cluster(cells[cid]);  // list full: this lane sums it
            }
            ncl += __popc(bal);
        }
        __syncwarp();
        warp_near_triangles(t9, cells, tri, p, cl_ids[wib], cl_pre[wib], min(ncl, kNearClCap), lane, s, c, mag, amb);
        float tot = s - c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
            err += __shfl_xor_sync(0xffffffffu, err, o);
            mag += __shfl_xor_sync(0xffffffffu, mag, o);
        }
        amb = __any_sync(0xffffffffu, amb);
        if (lane == 0) {
            const float w = fabsf(tot * kInv4Pi);
            const float E = (err + kFwnSlackRel * mag) * kInv4Pi + kFwnSlackAbs;
            if (!amb && w - E >= 0.5f) {
                consume(L, v, true, consumer, sbits, ds);
                ++certified;
            } else if (!amb && w + E < 0.5f) {
                consume(L, v, false, consumer, sbits, ds);
                ++certified;
            } else {
                const unsigned long long k = atomicAdd(&ds->fwn_fallback2, 1ull);
                if ((long long)k < fb_cap) fb2[k] = v;
            }
        }
    }
    if (lane == 0 && certified) atomicAdd(&ds->fwn_certified, certified);
}

// the next stage takes the leftovers of the last as its list
__global__ void fwn_handoff_kernel(DevState* ds, int only_if, long long fb_cap, unsigned long long* fb_n) {
    if (only_if && !ds->patching) return;
    ds->listed = min(*fb_n, (unsigned long long)fb_cap);
    *fb_n = 0ull;
}

constexpr int kRecheckThreads = 256;

// FP64 re-checks: each listed voxel's winding number summed in FP64 over every triangle.
// A short list (the usual case) would leave most SMs idle with one CTA per voxel, so each
// voxel's triangles are cut into S fixed slices (S up to 32, as many as the list buffer
// holds partial sums for: they go behind the n entries), one CTA per (voxel, slice), and a
// second kernel adds each voxel's S partials in slice order -- the sums do not depend on
// the launch. A long list runs one CTA per voxel.
__device__ __forceinline__ int recheck_slices(long long n, long long cap) {
    if (n <= 0) return 1;
    const long long s = (cap - n) / n;
    return (int)max(1LL, min(32LL, s));
}

__global__ void __launch_bounds__(kRecheckThreads) gwn_recheck_kernel(const float* __restrict__ tri9, long long T,
                                                                      Lattice L, long long* __restrict__ recheck,
                                                                      long long cap, int consumer,
                                                                      uint32_t* __restrict__ sbits, DevState* ds) {
    __shared__ double red[kRecheckThreads];
    const long long n = min((long long)ds->recheck_n, cap);
    const int S = recheck_slices(n, cap);
    double* partial = reinterpret_cast<double*>(recheck + n);
    for (long long e = blockIdx.x; e < n * S; e += gridDim.x) {
        const long long v = recheck[e / S];
        const long long sl = e % S;
        const long long t0 = T * sl / S, t1 = T * (sl + 1) / S;
        int x, y, z;
        voxel_coords(L, v, x, y, z);
        f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
        double s = 0.0;
        for (long long t = t0 + threadIdx.x; t < t1; t += kRecheckThreads) {
            const float* q = tri9 + t * 9;
            s += solid_angle_f64(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int o = kRecheckThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (S == 1) {
                double w = red[0] / (4.0 * 3.14159265358979323846);
                consume(L, v, fabs(w) >= 0.5, consumer, sbits, ds);
                atomicAdd(&ds->fp64_rechecks, 1ull);
            } else {
                partial[e] = red[0];
            }
        }
        __syncthreads();
    }
}

__global__ void gwn_recheck_final_kernel(Lattice L, const long long* __restrict__ recheck, long long cap,
                                         int consumer, uint32_t* __restrict__ sbits, DevState* ds) {
    const long long n = min((long long)ds->recheck_n, cap);
    const int S = recheck_slices(n, cap);
    if (S == 1) return;
    const double* partial = reinterpret_cast<const double*>(recheck + n);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < S; ++k) s += partial[i * S + k];
        const double w = s / (4.0 * 3.14159265358979323846);
        consume(L, recheck[i], fabs(w) >= 0.5, consumer, sbits, ds);
        atomicAdd(&ds->fp64_rechecks, 1ull);
    }
}

__global__ void verify_prepare_kernel(Lattice L, int gen, const uint32_t* __restrict__ ubits,
                                      long long* __restrict__ list, DevState* ds) {
    __shared__ int state;
    if (threadIdx.x == 0) state = ds->verify_state;
    __syncthreads();
    if (state != 0) {
        if (threadIdx.x == 0) ds->listed = 0;
        return;
    }
    const double off = (gen == 0) ? 0.5 : (gen == 1) ? (1.0 / 6.0) : (5.0 / 6.0);
    const unsigned long long N = (unsigned long long)L.N;
    for (int i = threadIdx.x; i < kVerifySamples; i += blockDim.x) {
        // cuda_rasterizer.cu:582-585
        unsigned long long v = (unsigned long long)(((double)i + off) * (double)N / (double)kVerifySamples);
        if (v >= N) v = N - 1;
        int x, y, z;
        voxel_coords(L, (long long)v, x, y, z);
        bool unknown = (ubits[word_of(L, x, y, z)] >> (x & 31)) & 1u;  // sign == 2 -> skipped (:588)
        list[i] = unknown ? -1 : (long long)v;
    }
    if (threadIdx.x == 0) {
        ds->patching = 0;
        ds->probe_m = 0;
        ds->recheck_n = 0;
        ds->listed = kVerifySamples;
    }
}

__global__ void verify_plan_kernel(int gen, DevState* ds, int escalate) {
    if (ds->verify_state != 0) return;
    int m = ds->probe_m;
    ds->probes += 1;
    if (m == 0) {
        ds->verify_state = 1;
        return;
    }
    if (escalate) {  // learned mode: any mismatch re-decides the signs, no patch boxes
        ds->total_sites += m;
        ds->verify_state = 2;
        return;
    }
    if (m > kVerifySamples) m = kVerifySamples;
    if (m > kMaxSitesPerProbe || gen == kProbeGens - 1) {
        ds->verify_state = 2;
        return;
    }
    ds->patching = 1;
    ds->total_sites += m;
    ds->patch_rounds += 1;
    ds->listed = 0;
    ds->recheck_n = 0;
    ds->list_overflow = 0;
}

__global__ void patch_mark_kernel(Lattice L, uint32_t* __restrict__ ubits, DevState* ds) {
    if (!ds->patching) return;
    const int s = blockIdx.x;
    if (s >= ds->probe_m) return;
    const long long v = ds->sites[s];
    int cx, cy, cz;
    voxel_coords(L, v, cx, cy, cz);
    const int r = kPatchRadius;
    int x0 = max(cx - r, 0), y0 = max(cy - r, 0), z0 = max(cz - r, 0);
    int x1 = min(cx + r, L.dims[0] - 1), y1 = min(cy + r, L.dims[1] - 1), z1 = min(cz + r, L.dims[2] - 1);
    const int ny = y1 - y0 + 1, nz = z1 - z0 + 1;
    // one row (y, z) per thread iteration; set the row's x range bit by bit per word
    for (int k = threadIdx.x; k < ny * nz; k += blockDim.x) {
        int y = y0 + k % ny, z = z0 + k / ny;
        for (int xw = x0 >> 5; xw <= (x1 >> 5); ++xw) {
            int lo = max(x0, xw * 32) - xw * 32, hi = min(x1, xw * 32 + 31) - xw * 32;
            uint32_t mask = (hi == 31 ? 0xffffffffu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
            atomicOr(&ubits[((size_t)z * L.dims[1] + y) * L.wx + xw], mask);
        }
    }
}

}  // namespace

void launch_list_unknown(uint32_t* ubits, uint32_t* sbits, const Lattice& L, long long* list, long long cap,
                         DevState* ds, int only_if_patching, cudaStream_t st, uint32_t* ebits) {
    long long blocks = std::min<long long>((L.nwords + 255) / 256, 152LL * 16);
    if (blocks < 1) blocks = 1;
    GBSDF_COUNT_LAUNCH();
    list_unknown_kernel<<<(unsigned)blocks, 256, 0, st>>>(ubits, sbits, ebits, L, list, cap, ds, only_if_patching);
}

void launch_gwn(const float* tri9, long long T, const Lattice& L, const long long* list, long long list_cap,
                int consumer, int only_if, uint32_t* sbits, long long* recheck, long long recheck_cap,
                const float* dist, int dist_sq, float surf_tol_vox, DevState* ds, int num_sms, cudaStream_t st) {
    // consumer kGwnVerify lists are short (<= 4096): one voxel per warp.
    if (consumer == kGwnVerify) {
        long long blocks = (kVerifySamples + 7) / 8;
        GBSDF_COUNT_LAUNCH();
        gwn_kernel<32><<<(unsigned)blocks, kGwnThreads, 0, st>>>(tri9, T, L, list, list_cap, consumer, only_if,
                                                                 sbits, recheck, recheck_cap, dist, dist_sq, surf_tol_vox, ds);
    } else {
        long long blocks = (long long)num_sms * 8;
        GBSDF_COUNT_LAUNCH();
        gwn_kernel<1><<<(unsigned)blocks, kGwnThreads, 0, st>>>(tri9, T, L, list, list_cap, consumer, only_if,
                                                                sbits, recheck, recheck_cap, dist, dist_sq, surf_tol_vox, ds);
    }
}

void launch_gwn_team(const float* tri9, long long T, const Lattice& L, long long* list, long long list_cap,
                     int consumer, uint32_t* sbits, long long* recheck, long long recheck_cap, const float* dist,
                     int dist_sq, float surf_tol_vox, DevState* ds, int num_sms, cudaStream_t st, int only_if) {
    GBSDF_COUNT_LAUNCH();
    gwn_sliced_kernel<<<(unsigned)(num_sms * 8), kGwnThreads, 0, st>>>(tri9, T, L, list, list_cap, consumer, only_if,
                                                                         sbits, recheck, recheck_cap, dist, dist_sq,
                                                                         surf_tol_vox, ds);
    GBSDF_COUNT_LAUNCH();
    gwn_sliced_final_kernel<<<16, 256, 0, st>>>(T, L, list, list_cap, consumer, only_if, sbits, recheck, recheck_cap,
                                                ds);
}

FwnGrid fwn_grid(const Lattice& L, long long T) {
    FwnGrid g{};
    int s = 8;
    auto cells_at = [&](int side) {
        long long c = 1;
        for (int k = 0; k < 3; ++k) c *= (L.dims[k] + side - 1) / side;
        return c;
    };
    while (s > 2 && T > 16 * cells_at(s)) s /= 2;
    g.s = s;
    for (int k = 0; k < 3; ++k) g.n[k] = (L.dims[k] + s - 1) / s;
    g.cells = cells_at(s);
    return g;
}

long long fwn_scan_elems(const FwnGrid& g) { return scan_tmp_elems(g.cells); }

void launch_fwn_build(const float* tri9, long long T, const Lattice& L, const Fwn& f, DevState* ds, cudaStream_t st) {
    if (T <= 0) return;
    const long long nc = f.g.cells;
    cudaMemsetAsync(f.counts, 0, (size_t)nc * 4, st);
    cudaMemsetAsync(f.cursor, 0, (size_t)nc * 4, st);
    GBSDF_COUNT_LAUNCH();
    fwn_count_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(tri9, T, L, f.g, f.cell_of, f.counts);
    launch_exclusive_scan(f.counts, f.off, nc, f.scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    fwn_flag_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(f.counts, nc, f.flag);
    launch_exclusive_scan(f.flag, f.cidx, nc, f.scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    fwn_fill_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(T, f.cell_of, f.off, f.cursor, f.tri);
    GBSDF_COUNT_LAUNCH();
    fwn_stats_kernel<<<(unsigned)((nc * 32 + 255) / 256), 256, 0, st>>>(tri9, nc, f.counts, f.off, f.flag, f.cidx,
                                                                        f.tri, f.cells, ds, f.g, f.sn[0], f.sn[1],
                                                                        f.sup_of);
    if (!f.supers) return;
    const long long ns = f.scells;
    cudaMemsetAsync(f.sup_counts, 0, (size_t)ns * 4, st);
    cudaMemsetAsync(f.sup_cursor, 0, (size_t)ns * 4, st);
    GBSDF_COUNT_LAUNCH();
    fwn_sup_count_kernel<<<152 * 4, 256, 0, st>>>(ds, f.sup_of, f.sup_counts);
    launch_exclusive_scan(f.sup_counts, f.sup_off, ns, f.scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    fwn_flag_kernel<<<(unsigned)((ns + 255) / 256), 256, 0, st>>>(f.sup_counts, ns, f.sup_flag);
    launch_exclusive_scan(f.sup_flag, f.sup_cidx, ns, f.scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    fwn_sup_fill_kernel<<<152 * 4, 256, 0, st>>>(ds, f.sup_of, f.sup_off, f.sup_cursor, f.sup_child);
    GBSDF_COUNT_LAUNCH();
    fwn_sup_stats_kernel<<<(unsigned)((ns * 32 + 255) / 256), 256, 0, st>>>(
        ns, f.sup_counts, f.sup_off, f.sup_flag, f.sup_cidx, f.sup_child, f.cells, f.supers, ds);
}

size_t fwn_super_bytes(const FwnGrid& g, long long T, long long cap) {
    long long ns = 1;
    for (int k = 0; k < 3; ++k) ns *= (g.n[k] + 3) / 4;
    const long long ncap = std::max<long long>(1, std::min<long long>(g.cells, T));
    const long long scap = std::max<long long>(1, std::min<long long>(ns, ncap));
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    return al(scap * sizeof(FwnCell)) + al(ncap * 4) + 3 * al(ns * 4) + 2 * al(ns * 8) + al(ncap * 4) + al(cap * 8);
}

void fwn_super_carve(Fwn& f, void* base, long long T, long long cap) {
    long long ns = 1;
    for (int k = 0; k < 3; ++k) {
        f.sn[k] = (f.g.n[k] + 3) / 4;
        ns *= f.sn[k];
    }
    f.scells = ns;
    const long long ncap = std::max<long long>(1, std::min<long long>(f.g.cells, T));
    const long long scap = std::max<long long>(1, std::min<long long>(ns, ncap));
    char* p = static_cast<char*>(base);
    auto take = [&](size_t b) {
        char* q = p;
        p += (b + 255) & ~size_t(255);
        return q;
    };
    f.supers = reinterpret_cast<FwnCell*>(take(scap * sizeof(FwnCell)));
    f.sup_of = reinterpret_cast<unsigned*>(take(ncap * 4));
    f.sup_counts = reinterpret_cast<unsigned*>(take(ns * 4));
    f.sup_cursor = reinterpret_cast<unsigned*>(take(ns * 4));
    f.sup_flag = reinterpret_cast<unsigned*>(take(ns * 4));
    f.sup_off = reinterpret_cast<unsigned long long*>(take(ns * 8));
    f.sup_cidx = reinterpret_cast<unsigned long long*>(take(ns * 8));
    f.sup_child = reinterpret_cast<unsigned*>(take(ncap * 4));
    f.fb2 = reinterpret_cast<long long*>(take(cap * 8));
}

void launch_winding(const Fwn* f, const float* tri9, long long T, const Lattice& L, const long long* list,
                    long long list_cap, int consumer, int only_if, uint32_t* sbits, long long* recheck,
                    long long recheck_cap, const float* dist, int dist_sq, float surf_tol_vox, DevState* ds,
                    int num_sms, cudaStream_t st) {
    if (!f) {
        launch_gwn(tri9, T, L, list, list_cap, consumer, only_if, sbits, recheck, recheck_cap, dist, dist_sq,
                   surf_tol_vox, ds, num_sms, st);
        return;
    }
    // stages, each taking the voxels the last could not decide: super-clusters (when built),
    // clusters at beta, clusters at kFwnBetaFine (smaller truncation bounds, more triangles
    // summed near the voxel), then the per-triangle sum
    long long* bufs[2] = {f->fb2, f->fb};
    long long* left = nullptr;  // the last stage's leftovers
    int nb = 0;
    if (f->supers) {
        GBSDF_COUNT_LAUNCH();
        fwn_query_sup_kernel<<<(unsigned)(num_sms * 8), kGwnThreads, 0, st>>>(
            tri9, f->cells, f->tri, f->supers, f->sup_child, L, list, list_cap, consumer, only_if, sbits, dist,
            dist_sq, surf_tol_vox, ds, bufs[0], f->fb_cap);
        GBSDF_COUNT_LAUNCH();
        fwn_handoff_kernel<<<1, 1, 0, st>>>(ds, only_if, f->fb_cap, &ds->fwn_fallback2);
        list = bufs[0];
        list_cap = f->fb_cap;
        nb = 1;
    }
    const float betas[2] = {kFwnBeta, kFwnBetaFine};
    // the refining stage pays off when the per-triangle sum it spares is long
    const int stages = (T >= kFwnFineMinTris) ? 2 : 1;
    for (int stg = 0; stg < stages; ++stg) {
        long long* out = f->fb2 ? bufs[nb & 1] : f->fb;
        unsigned long long* cnt = (nb & 1) ? &ds->fwn_fallback : &ds->fwn_fallback2;
        if (!f->fb2) cnt = &ds->fwn_fallback;
        GBSDF_COUNT_LAUNCH();
        fwn_query_kernel<<<(unsigned)(num_sms * 8), kGwnThreads, 0, st>>>(
            tri9, f->cells, f->tri, L, list, list_cap, consumer, only_if, sbits, dist, dist_sq, surf_tol_vox, ds, out,
            f->fb_cap, betas[stg], cnt, stg == stages - 1 || !f->fb2);
        GBSDF_COUNT_LAUNCH();
        fwn_handoff_kernel<<<1, 1, 0, st>>>(ds, only_if, f->fb_cap, cnt);
        list = out;
        left = out;
        list_cap = f->fb_cap;
        ++nb;
        if (!f->fb2) break;  // one buffer: a single cluster stage
    }
    launch_gwn_team(tri9, T, L, left, f->fb_cap, consumer, sbits, recheck, recheck_cap, dist, dist_sq, surf_tol_vox,
                    ds, num_sms, st, only_if);
}

void launch_gwn_small(const float* tri9, long long T, const Lattice& L, const long long* list, long long list_cap,
                      int consumer, uint32_t* sbits, long long* recheck, long long recheck_cap, const float* dist,
                      int dist_sq, float surf_tol_vox, DevState* ds, long long n_hint, cudaStream_t st) {
    long long blocks = std::max<long long>(1, (n_hint + 7) / 8);
    GBSDF_COUNT_LAUNCH();
    gwn_kernel<32><<<(unsigned)blocks, kGwnThreads, 0, st>>>(tri9, T, L, list, list_cap, consumer, 0, sbits,
                                                             recheck, recheck_cap, dist, dist_sq, surf_tol_vox, ds);
}

void launch_gwn_recheck(const float* tri9, long long T, const Lattice& L, long long* recheck,
                        long long recheck_cap, int consumer, uint32_t* sbits, DevState* ds, int num_sms,
                        cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    gwn_recheck_kernel<<<(unsigned)(num_sms * 4), kRecheckThreads, 0, st>>>(tri9, T, L, recheck, recheck_cap,
                                                                          consumer, sbits, ds);
    GBSDF_COUNT_LAUNCH();
    gwn_recheck_final_kernel<<<16, 256, 0, st>>>(L, recheck, recheck_cap, consumer, sbits, ds);
}

void launch_verify_prepare(const Lattice& L, int gen, const uint32_t* ubits, long long* list, DevState* ds,
                           cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    verify_prepare_kernel<<<1, 1024, 0, st>>>(L, gen, ubits, list, ds);
}

void launch_verify_plan(int gen, DevState* ds, cudaStream_t st, int escalate) {
    GBSDF_COUNT_LAUNCH();
    verify_plan_kernel<<<1, 1, 0, st>>>(gen, ds, escalate);
}

void launch_patch_mark(const Lattice& L, uint32_t* ubits, DevState* ds, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    patch_mark_kernel<<<kMaxSitesPerProbe, 256, 0, st>>>(L, ubits, ds);
}

}  // namespace gbsdf
