// k_splat.cu — triangle preparation, brick / strip binning (counting sort) and
// the exact band splat [A] of the mesh-to-SDF path.
//
// The reference splats with one thread per (triangle, z-layer) and a CAS-loop
// atomicMin into the grid (cuda_rasterizer.cu:211-268). Here each triangle is
// binned to the 8^3 bricks its clamped footprint touches; one CTA owns one brick,
// stages the brick's triangle list in shared memory and keeps each voxel's
// minimum in registers, so the grid sees one plain store per band voxel and no
// atomics. The per-(voxel, triangle) predicates are the reference's own: the
// z-layer test, the clamped integer XY footprint, the AABB box test and
// d^2 <= band^2 (cuda_rasterizer.cu:225-266), so the set of candidate distances of
// every voxel -- and therefore its minimum -- is the reference's.
#include <algorithm>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

constexpr int kPrepThreads = 256;

__device__ __forceinline__ bool finite3(f3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

// Conservative plane test between a brick and a triangle's band: the plane
// distance from the brick centre lower-bounds the distance of every brick voxel
// to the triangle, so a brick whose centre is farther than band + half-diagonal
// (+ a relative margin far above FP32 rounding) can hold no band voxel of it.
__device__ __forceinline__ bool brick_may_hit(const SplatTri& r, const Lattice& L, int bx, int by, int bz,
                                              float bw) {
    float h = L.h;
    float cx = ((float)(L.mn[0] + bx * kBrick) + 3.5f) * h;
    float cy = ((float)(L.mn[1] + by * kBrick) + 3.5f) * h;
    float cz = ((float)(L.mn[2] + bz * kBrick) + 3.5f) * h;
    float ex = r.v[3] - r.v[0], ey = r.v[4] - r.v[1], ez = r.v[5] - r.v[2];
    float fx = r.v[6] - r.v[0], fy = r.v[7] - r.v[1], fz = r.v[8] - r.v[2];
    float nx = ey * fz - ez * fy, ny = ez * fx - ex * fz, nz = ex * fy - ey * fx;
    float nn = nx * nx + ny * ny + nz * nz;
    if (!(nn > 1e-30f)) return true;
    float dist = fabsf(nx * (cx - r.v[0]) + ny * (cy - r.v[1]) + nz * (cz - r.v[2])) * rsqrtf(nn);
    float reach = bw + 6.0621778f * h * 1.0001f + 1e-3f * (bw + 7.0f * h) + 1e-4f * fabsf(dist);
    return dist <= reach;
}

__global__ void __launch_bounds__(kPrepThreads) prep_kernel(const float* __restrict__ tris12, long long T,
                                                            Lattice L, SplatTri* __restrict__ sto,
                                                            ParTri* __restrict__ pto,
                                                            unsigned* __restrict__ brick_count,
                                                            unsigned* __restrict__ strip_count, DevState* ds) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float* r = tris12 + 12 * t;
    f3 v0 = mk(r[0], r[1], r[2]), v1 = mk(r[3], r[4], r[5]), v2 = mk(r[6], r[7], r[8]);
    const float h = L.h;
    const float bw = (float)kBandVoxels * h;
    SplatTri s;
    ParTri p;
    for (int k = 0; k < 3; ++k) {
        s.v[k] = r[k];
        s.v[3 + k] = r[3 + k];
        s.v[6 + k] = r[6 + k];
        p.v[k] = r[k];
        p.v[3 + k] = r[3 + k];
        p.v[6 + k] = r[6 + k];
    }
    s.valid = 0;
    s.pad[0] = s.pad[1] = 0;
    p.sx0 = 0;
    p.sx1 = -1;
    p.sy0 = 0;
    p.sy1 = -1;
    p.pad[0] = p.pad[1] = p.pad[2] = 0;
    // FP64 bounds validation before any float->int grid arithmetic.
    bool ok = finite3(v0) && finite3(v1) && finite3(v2);
    if (ok) {
        const double lim = 1.0e9;
        double hd = (double)h;
        const float* vv = r;
        for (int k = 0; k < 9; ++k) {
            double c = (double)vv[k] / hd;
            if (!(fabs(c) < lim)) ok = false;
        }
    }
    if (!ok) {
        atomicAdd(&ds->invalid_tris, 1ull);
        for (int k = 0; k < 6; ++k) s.bb[k] = 0.0f;
        s.fx0 = s.fy0 = s.z0 = 0;
        s.fx1 = s.fy1 = s.z1 = -1;
        for (int k = 0; k < 4; ++k) p.xyab[k] = 0.0f;
        sto[t] = s;
        pto[t] = p;
        return;
    }
    // ---- splat footprint, cuda_rasterizer.cu:225-248
    float tx0 = fminf(v0.x, fminf(v1.x, v2.x)), tx1 = fmaxf(v0.x, fmaxf(v1.x, v2.x));
    float ty0 = fminf(v0.y, fminf(v1.y, v2.y)), ty1 = fmaxf(v0.y, fmaxf(v1.y, v2.y));
    float tz0 = fminf(v0.z, fminf(v1.z, v2.z)), tz1 = fmaxf(v0.z, fmaxf(v1.z, v2.z));
    s.bb[0] = tx0;
    s.bb[1] = tx1;
    s.bb[2] = ty0;
    s.bb[3] = ty1;
    s.bb[4] = tz0;
    s.bb[5] = tz1;
    int x0 = (int)ceilf((tx0 - bw) / h) - L.mn[0];
    int x1 = (int)floorf((tx1 + bw) / h) - L.mn[0];
    int y0 = (int)ceilf((ty0 - bw) / h) - L.mn[1];
    int y1 = (int)floorf((ty1 + bw) / h) - L.mn[1];
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (x1 > L.dims[0] - 1) x1 = L.dims[0] - 1;
    if (y1 > L.dims[1] - 1) y1 = L.dims[1] - 1;
    // conservative z range; the exact per-layer test runs per voxel in the splat
    int z0 = (int)floorf((tz0 - bw) / h) - L.mn[2] - 1;
    int z1 = (int)ceilf((tz1 + bw) / h) - L.mn[2] + 1;
    if (z0 < 0) z0 = 0;
    if (z1 > L.dims[2] - 1) z1 = L.dims[2] - 1;
    s.fx0 = x0;
    s.fx1 = x1;
    s.fy0 = y0;
    s.fy1 = y1;
    s.z0 = z0;
    s.z1 = z1;
    s.valid = (x1 >= x0 && y1 >= y0 && z1 >= z0) ? 1 : 0;
    if (s.valid) {
        unsigned long long pairs = 0;
        for (int bz = z0 / kBrick; bz <= z1 / kBrick; ++bz)
            for (int by = y0 / kBrick; by <= y1 / kBrick; ++by)
                for (int bx = x0 / kBrick; bx <= x1 / kBrick; ++bx) {
                    if (!brick_may_hit(s, L, bx, by, bz, bw)) continue;
                    atomicAdd(&brick_count[((long long)bz * L.nb[1] + by) * L.nb[0] + bx], 1u);
                    ++pairs;
                }
        atomicAdd(&ds->brick_pairs, pairs);
    }
    sto[t] = s;
    // ---- parity record: the reference's host CSR coverage, cuda_rasterizer.cu:837-860
    float minx = fminf(v0.x, fminf(v1.x, v2.x)), maxx = fmaxf(v0.x, fmaxf(v1.x, v2.x));
    float miny = fminf(v0.y, fminf(v1.y, v2.y)), maxy = fmaxf(v0.y, fmaxf(v1.y, v2.y));
    p.xyab[0] = minx;
    p.xyab[1] = miny;
    p.xyab[2] = maxx;
    p.xyab[3] = maxy;
    int sdx = (L.dims[0] + kSup - 1) / kSup, sdy = (L.dims[1] + kSup - 1) / kSup;
    int cx0 = (int)floorf(minx / h) - L.mn[0] - 1;
    int cx1 = (int)ceilf(maxx / h) - L.mn[0] + 1;
    int cy0 = (int)floorf(miny / h) - L.mn[1] - 1;
    int cy1 = (int)ceilf(maxy / h) - L.mn[1] + 1;
    int sx0 = max(0, cx0 / kSup), sx1 = min(sdx - 1, cx1 / kSup);
    int sy0 = max(0, cy0 / kSup), sy1 = min(sdy - 1, cy1 / kSup);
    p.sx0 = sx0;
    p.sx1 = sx1;
    p.sy0 = sy0;
    p.sy1 = sy1;
    pto[t] = p;
    if (sx1 >= sx0 && sy1 >= sy0) {
        atomicAdd(&ds->csr_entries, (unsigned long long)(sx1 - sx0 + 1) * (unsigned long long)(sy1 - sy0 + 1));
        int xa = sx0 * kSup, xb = min(L.dims[0] - 1, sx1 * kSup + kSup - 1);
        int ya = sy0 * kSup, yb = min(L.dims[1] - 1, sy1 * kSup + kSup - 1);
        unsigned long long pairs = 0;
        for (int y = ya; y <= yb; ++y)
            for (int sx = xa / kStrip; sx <= xb / kStrip; ++sx) {
                atomicAdd(&strip_count[(long long)y * L.nsx + sx], 1u);
                ++pairs;
            }
        atomicAdd(&ds->strip_pairs, pairs);
    }
}

__global__ void __launch_bounds__(kPrepThreads) bin_fill_kernel(
    const SplatTri* __restrict__ stt, const ParTri* __restrict__ ptt, long long T, Lattice L,
    const unsigned long long* __restrict__ brick_off, unsigned* __restrict__ brick_cur,
    unsigned* __restrict__ brick_list, const unsigned long long* __restrict__ strip_off,
    unsigned* __restrict__ strip_cur, unsigned* __restrict__ strip_list, DevState* ds, unsigned long long cap_b,
    unsigned long long cap_s) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    if (ds && (ds->brick_pairs > cap_b || ds->strip_pairs > cap_s)) {  // planned lists too small
        if (t == 0) ds->overflow = 1;
        return;
    }
    const float bw = (float)kBandVoxels * L.h;
    SplatTri s = stt[t];
    if (s.valid) {
        for (int bz = s.z0 / kBrick; bz <= s.z1 / kBrick; ++bz)
            for (int by = s.fy0 / kBrick; by <= s.fy1 / kBrick; ++by)
                for (int bx = s.fx0 / kBrick; bx <= s.fx1 / kBrick; ++bx) {
                    if (!brick_may_hit(s, L, bx, by, bz, bw)) continue;
                    long long b = ((long long)bz * L.nb[1] + by) * L.nb[0] + bx;
                    unsigned pos = atomicAdd(&brick_cur[b], 1u);
                    brick_list[brick_off[b] + pos] = (unsigned)t;
                }
    }
    ParTri p = ptt[t];
    if (p.sx1 >= p.sx0 && p.sy1 >= p.sy0) {
        int xa = p.sx0 * kSup, xb = min(L.dims[0] - 1, p.sx1 * kSup + kSup - 1);
        int ya = p.sy0 * kSup, yb = min(L.dims[1] - 1, p.sy1 * kSup + kSup - 1);
        for (int y = ya; y <= yb; ++y)
            for (int sx = xa / kStrip; sx <= xb / kStrip; ++sx) {
                long long b = (long long)y * L.nsx + sx;
                unsigned pos = atomicAdd(&strip_cur[b], 1u);
                strip_list[strip_off[b] + pos] = (unsigned)t;
            }
    }
}

// ---- exclusive scan (unsigned -> unsigned long long), three-phase, recursive on the host
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

template <typename Tin>
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const Tin* __restrict__ in,
                                                                 unsigned long long* __restrict__ out, long long n,
                                                                 unsigned long long* __restrict__ tile_sums) {
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned long long v[kScanItems];
    unsigned long long run = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        long long k = base + i;
        unsigned long long x = (k < n) ? (unsigned long long)in[k] : 0ull;
        v[i] = run;
        run += x;
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned long long wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += warp_tot[w];
    unsigned long long excl = wpre + incl - run;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        long long k = base + i;
        if (k < n) out[k] = v[i] + excl;
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = wpre + incl;
}

__global__ void scan_add_kernel(unsigned long long* __restrict__ out, long long n,
                                const unsigned long long* __restrict__ tile_off) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] += tile_off[k / kScanTile];
}

void scan_rec(const void* in, bool in_is_u64, unsigned long long* out, long long n, unsigned long long* tmp,
              cudaStream_t st) {
    long long tiles = (n + kScanTile - 1) / kScanTile;
    unsigned long long* sums = tmp;
    unsigned long long* rest = tmp + tiles;
    GBSDF_COUNT_LAUNCH();
    if (in_is_u64)
        scan_tile_kernel<unsigned long long><<<(unsigned)tiles, kScanThreads, 0, st>>>(
            (const unsigned long long*)in, out, n, sums);
    else
        scan_tile_kernel<unsigned><<<(unsigned)tiles, kScanThreads, 0, st>>>((const unsigned*)in, out, n, sums);
    if (tiles > 1) {
        unsigned long long* sums_scanned = rest;
        scan_rec(sums, true, sums_scanned, tiles, rest + tiles, st);
        GBSDF_COUNT_LAUNCH();
        scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, sums_scanned);
    }
}

constexpr int kSplatThreads = 128;
constexpr int kSplatChunk = 64;

// The bricks with binned triangles: those with at most `dense_cut` from the front of
// `active` (ds->active_bricks of them, splat_kernel's), the others from the back
// (ds->dense_bricks, splat_dense_kernel's).
__global__ void active_bricks_kernel(const unsigned* __restrict__ cnt, long long nb, unsigned* __restrict__ active,
                                     DevState* ds, unsigned dense_cut) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned n = (b < nb) ? cnt[b] : 0u;
    const bool sparse = n > 0 && n <= dense_cut, dense = n > dense_cut;
    const unsigned ms = __ballot_sync(0xffffffffu, sparse), md = __ballot_sync(0xffffffffu, dense);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    unsigned long long bs = 0, bd = 0;
    if (lane == 0) {
        if (ms) bs = atomicAdd(&ds->active_bricks, (unsigned long long)__popc(ms));
        if (md) bd = atomicAdd(&ds->dense_bricks, (unsigned long long)__popc(md));
    }
    bs = __shfl_sync(0xffffffffu, bs, 0);
    bd = __shfl_sync(0xffffffffu, bd, 0);
    if (sparse) active[bs + __popc(ms & below)] = (unsigned)b;
    if (dense) active[nb - 1 - (long long)(bd + __popc(md & below))] = (unsigned)b;
}

__global__ void fill_kernel(float4* __restrict__ g4, long long n4, float value) {
    long long stride = (long long)gridDim.x * blockDim.x;
    float4 v = make_float4(value, value, value, value);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) g4[i] = v;
}
__global__ void fill_tail_kernel(float* __restrict__ g, long long from, long long n, float value) {
    long long i = from + threadIdx.x;
    if (i < n) g[i] = value;
}


// One staged triangle against one thread's K voxels (x, y, wz[k]). CULL: skip a triangle
// whose bounding-box distance^2 exceeds the voxel's best exact distance^2 by more than both
// computations' rounding (a few ulps of the largest coordinate), which cannot lower the
// minimum -- the result stays bit-identical.
template <bool CULL, int K>
__device__ __forceinline__ void splat_tri(const SplatTri& r, int x, int y, float px, float py, const float (&wz)[K],
                                          float bw, float band_sq, float (&best)[K], unsigned& evals) {
    if (x < r.fx0 || x > r.fx1 || y < r.fy0 || y > r.fy1) return;
    const float tx0 = r.bb[0], tx1 = r.bb[1], ty0 = r.bb[2], ty1 = r.bb[3], tz0 = r.bb[4], tz1 = r.bb[5];
    const float bdx = (px < tx0) ? (tx0 - px) : ((px > tx1) ? (px - tx1) : 0.0f);
    const float bdy = (py < ty0) ? (ty0 - py) : ((py > ty1) ? (py - ty1) : 0.0f);
    const float bxy = bdx * bdx + bdy * bdy;
    const f3 a = mk(r.v[0], r.v[1], r.v[2]), bb = mk(r.v[3], r.v[4], r.v[5]), c = mk(r.v[6], r.v[7], r.v[8]);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float z = wz[k];
        if (z < tz0 - bw || z > tz1 + bw) continue;
        const float bdz = (z < tz0) ? (tz0 - z) : ((z > tz1) ? (z - tz1) : 0.0f);
        const float lb = bxy + bdz * bdz;
        if (lb > band_sq) continue;
        if constexpr (CULL) {
            if (best[k] < band_sq) {
                const float sc = fmaxf(fmaxf(fmaxf(fabsf(px), fabsf(py)), fmaxf(fabsf(tx0), fabsf(tx1))),
                                       fmaxf(fmaxf(fabsf(ty0), fabsf(ty1)), fmaxf(fabsf(tz0), fabsf(tz1))));
                const float dz = fmaxf(sc, fabsf(z)) * 3.814697265625e-6f;  // 2^-18 of the magnitude
                const float margin = 4.0f * dz * (sqrtf(best[k]) + dz) + best[k] * 1e-5f;
                if (lb > best[k] + margin) continue;
            }
        }
        const float d2 = ptd_sq(mk(px, py, z), a, bb, c);
        ++evals;
        if (d2 <= band_sq && d2 < best[k]) best[k] = d2;
    }
}

// ---- dense bricks: per-sub-brick triangle lists ----------------------------------------
// A brick with more than the tile cut's binned triangles is split into its eight 4^3
// sub-bricks, one warp each (a lane owns 2 voxels of one column). A first pass over the
// brick's list finds the sub-brick centre's nearest triangle T*: every lattice point v of
// the sub-brick has d(v, T*) <= d(centre, T*) + R (R the half-diagonal of the sub-brick's
// point box), so a triangle whose bounding box is farther than that from the point box
// cannot be nearer than T* to any of its voxels. The second pass stages the list again and
// each warp keeps, per chunk, only the triangles that pass this test (widened by 16 x 2^-18
// of the coordinate magnitude for the rounding of both sides), then runs the per-voxel
// update on them. Skipped triangles never hold a voxel's minimum, so the distances are the
// sparse kernel's, bit for bit; the screening work drops from 512 voxel tests per triangle
// to 8 exact distances plus the survivors' tests.
constexpr int kDenseThreads = 256;
constexpr int kDenseSlices = 8;  // CTAs per dense brick, each on an eighth of its triangle list

// One slice of one dense brick's list per CTA (grid: dense bricks x kDenseSlices, the
// bricks visited grid-stride). The slice's own nearest triangle to each sub-brick centre
// bounds the slice: a voxel's nearest triangle of the whole list is, within its slice,
// nearer than any other, so it survives its slice's test, and the minimum over the slices
// (an atomic minimum on the distance's bits, which order like unsigned integers for
// non-negative floats) is the whole list's. The band voxels of these bricks are counted
// afterwards by dense_count_kernel, once each.
__global__ void __launch_bounds__(kDenseThreads) splat_dense_kernel(
    const SplatTri* __restrict__ stt, const unsigned long long* __restrict__ off, const unsigned* __restrict__ cnt,
    const unsigned* __restrict__ list, const unsigned* __restrict__ active, Lattice L, float* __restrict__ dist,
    DevState* ds) {
    __shared__ SplatTri s[kSplatChunk];
    __shared__ unsigned char keep_idx[kDenseThreads / 32][kSplatChunk];
    if (ds->overflow) return;
    const unsigned long long nd = ds->dense_bricks;
    const int nbx = L.nb[0], nby = L.nb[1];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float h = L.h;
    const float bw = (float)kBandVoxels * h;
    const float band_sq = bw * bw;
    const int* src = reinterpret_cast<const int*>(stt);
    int* dsm = reinterpret_cast<int*>(s);
    unsigned evals = 0;
    for (unsigned long long di = blockIdx.x; di < nd; di += gridDim.x) {
        const unsigned b = active[L.nbricks - 1 - (long long)di];
        const unsigned n = cnt[b];
        const unsigned lo = (unsigned)((unsigned long long)n * blockIdx.y / kDenseSlices);
        const unsigned hi = (unsigned)((unsigned long long)n * (blockIdx.y + 1) / kDenseSlices);
        const int bx = (int)(b % (unsigned)nbx), by = (int)((b / (unsigned)nbx) % (unsigned)nby),
                  bz = (int)(b / ((unsigned)nbx * (unsigned)nby));
        const int x0 = bx * kBrick + (warp & 1) * 4, y0 = by * kBrick + ((warp >> 1) & 1) * 4,
                  z0 = bz * kBrick + (warp >> 2) * 4;
        const int x = x0 + (lane & 3), y = y0 + ((lane >> 2) & 3), zl = lane >> 4;
        const float px = (float)(L.mn[0] + x) * h, py = (float)(L.mn[1] + y) * h;
        float wz[2], best[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            wz[k] = (float)(L.mn[2] + z0 + zl + 2 * k) * h;
            best[k] = __int_as_float(0x7f800000);
        }
        // the sub-brick's point box (the lattice coordinates its voxels compute) and centre
        const float sx0 = (float)(L.mn[0] + x0) * h, sx1 = (float)(L.mn[0] + x0 + 3) * h;
        const float sy0 = (float)(L.mn[1] + y0) * h, sy1 = (float)(L.mn[1] + y0 + 3) * h;
        const float sz0 = (float)(L.mn[2] + z0) * h, sz1 = (float)(L.mn[2] + z0 + 3) * h;
        const f3 ctr = mk(0.5f * (sx0 + sx1), 0.5f * (sy0 + sy1), 0.5f * (sz0 + sz1));
        const float mag = fmaxf(fmaxf(fmaxf(fabsf(sx0), fabsf(sx1)), fmaxf(fabsf(sy0), fabsf(sy1))),
                                fmaxf(fabsf(sz0), fabsf(sz1))) + bw;
        const unsigned long long o = off[b];
        // pass 1: the centre's nearest triangle of the slice
        float u2 = __int_as_float(0x7f800000);
        for (unsigned c0 = lo; c0 < hi; c0 += kSplatChunk) {
            const unsigned m = min((unsigned)kSplatChunk, hi - c0);
            for (unsigned w = tid; w < m * 24u; w += kDenseThreads) {
                const unsigned rec = w / 24u, word = w - rec * 24u;
                dsm[w] = __ldg(src + (size_t)list[o + c0 + rec] * 24 + word);
            }
            __syncthreads();
            for (unsigned i = lane; i < m; i += 32) {
                const SplatTri& r = s[i];
                u2 = fminf(u2, ptd_sq(ctr, mk(r.v[0], r.v[1], r.v[2]), mk(r.v[3], r.v[4], r.v[5]),
                                      mk(r.v[6], r.v[7], r.v[8])));
            }
            __syncthreads();
        }
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) u2 = fminf(u2, __shfl_xor_sync(0xffffffffu, u2, sh));
        const float ex = sx1 - sx0, ey = sy1 - sy0, ez = sz1 - sz0;
        const float ub = sqrtf(u2) + 0.5f * sqrtf(ex * ex + ey * ey + ez * ez) + 16.0f * mag * 3.814697265625e-6f;
        const float ub2 = ub * ub;
        // pass 2: per chunk, this warp's surviving triangles, then the per-voxel update
        for (unsigned c0 = lo; c0 < hi; c0 += kSplatChunk) {
            const unsigned m = min((unsigned)kSplatChunk, hi - c0);
            for (unsigned w = tid; w < m * 24u; w += kDenseThreads) {
                const unsigned rec = w / 24u, word = w - rec * 24u;
                dsm[w] = __ldg(src + (size_t)list[o + c0 + rec] * 24 + word);
            }
            __syncthreads();
            unsigned nk = 0;
            for (unsigned base = 0; base < m; base += 32) {
                const unsigned i = base + lane;
                bool keep = false;
                if (i < m) {
                    const SplatTri& r = s[i];
                    if (!(x0 + 3 < r.fx0 || x0 > r.fx1 || y0 + 3 < r.fy0 || y0 > r.fy1)) {
                        const float gx = fmaxf(fmaxf(r.bb[0] - sx1, sx0 - r.bb[1]), 0.0f);
                        const float gy = fmaxf(fmaxf(r.bb[2] - sy1, sy0 - r.bb[3]), 0.0f);
                        const float gz = fmaxf(fmaxf(r.bb[4] - sz1, sz0 - r.bb[5]), 0.0f);
                        keep = gx * gx + gy * gy + gz * gz <= ub2;
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) keep_idx[warp][nk + __popc(bal & ((1u << lane) - 1u))] = (unsigned char)i;
                nk += __popc(bal);
            }
            __syncwarp();
            for (unsigned j = 0; j < nk; ++j)
                splat_tri<true, 2>(s[keep_idx[warp][j]], x, y, px, py, wz, bw, band_sq, best, evals);
            __syncthreads();
        }
        if (x < L.dims[0] && y < L.dims[1]) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int z = z0 + zl + 2 * k;
                if (z < L.dims[2] && best[k] != __int_as_float(0x7f800000))
                    atomicMin(reinterpret_cast<unsigned*>(dist) + ((size_t)z * L.dims[1] + y) * L.dims[0] + x,
                              __float_as_uint(sqrtf(best[k])));
            }
        }
    }
    const unsigned ew = __reduce_add_sync(0xffffffffu, evals);
    if (lane == 0 && ew) atomicAdd(&ds->splat_evals, (unsigned long long)ew);
}

// The band voxels of the dense bricks (the splat's atomic minima leave them below the far
// sentinel), counted once each.
__global__ void __launch_bounds__(256) dense_count_kernel(const unsigned* __restrict__ active, Lattice L,
                                                          const float* __restrict__ dist, DevState* ds) {
    if (ds->overflow) return;
    const unsigned long long nd = ds->dense_bricks;
    const int nbx = L.nb[0], nby = L.nb[1];
    unsigned found = 0;
    for (unsigned long long di = blockIdx.x; di < nd; di += gridDim.x) {
        const unsigned b = active[L.nbricks - 1 - (long long)di];
        const int bx = (int)(b % (unsigned)nbx), by = (int)((b / (unsigned)nbx) % (unsigned)nby),
                  bz = (int)(b / ((unsigned)nbx * (unsigned)nby));
        for (int v = threadIdx.x; v < kBrick * kBrick * kBrick; v += blockDim.x) {
            const int x = bx * kBrick + (v & 7), y = by * kBrick + ((v >> 3) & 7), z = bz * kBrick + (v >> 6);
            if (x < L.dims[0] && y < L.dims[1] && z < L.dims[2] &&
                dist[((size_t)z * L.dims[1] + y) * L.dims[0] + x] < kFarSentinel)
                ++found;
        }
    }
    const unsigned fw = __reduce_add_sync(0xffffffffu, found);
    if ((threadIdx.x & 31) == 0 && fw) atomicAdd(&ds->band_voxels, (unsigned long long)fw);
}

__global__ void __launch_bounds__(kSplatThreads) splat_kernel(
    const SplatTri* __restrict__ stt, const unsigned long long* __restrict__ off, const unsigned* __restrict__ cnt,
    const unsigned* __restrict__ list, const unsigned* __restrict__ active, Lattice L, float* __restrict__ dist,
    DevState* ds) {
    __shared__ SplatTri s[kSplatChunk];
    if (blockIdx.x >= ds->active_bricks || ds->overflow) return;
    const unsigned b = active[blockIdx.x];
    const int nbx = L.nb[0], nby = L.nb[1];
    const int bx = (int)(b % (unsigned)nbx), by = (int)((b / (unsigned)nbx) % (unsigned)nby),
              bz = (int)(b / ((unsigned)nbx * (unsigned)nby));
    const int tid = threadIdx.x;
    const int x = bx * kBrick + (tid & 7), y = by * kBrick + ((tid >> 3) & 7);
    const int zb = bz * kBrick + (tid >> 6);
    const float h = L.h;
    const float bw = (float)kBandVoxels * h;
    const float band_sq = bw * bw;
    const float px = (float)(L.mn[0] + x) * h, py = (float)(L.mn[1] + y) * h;
    float wz[4];
    float best[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        wz[k] = (float)(L.mn[2] + zb + 2 * k) * h;
        best[k] = __int_as_float(0x7f800000);  // +inf
    }
    const unsigned long long o = off[b];
    const unsigned n = cnt[b];
    unsigned evals = 0;
    for (unsigned c0 = 0; c0 < n; c0 += kSplatChunk) {
        unsigned m = min((unsigned)kSplatChunk, n - c0);
        // stage the chunk: m records x 24 words
        const int* src = reinterpret_cast<const int*>(stt);
        int* dsm = reinterpret_cast<int*>(s);
        for (unsigned w = tid; w < m * 24u; w += kSplatThreads) {
            unsigned rec = w / 24u, word = w - rec * 24u;
            unsigned t = list[o + c0 + rec];
            dsm[w] = __ldg(src + (size_t)t * 24 + word);
        }
        __syncthreads();
        for (unsigned i = 0; i < m; ++i) splat_tri<false, 4>(s[i], x, y, px, py, wz, bw, band_sq, best, evals);
        __syncthreads();
    }
    unsigned found = 0;
    if (x < L.dims[0] && y < L.dims[1]) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int z = zb + 2 * k;
            if (z < L.dims[2] && best[k] != __int_as_float(0x7f800000)) {
                size_t idx = ((size_t)z * L.dims[1] + y) * L.dims[0] + x;
                dist[idx] = sqrtf(best[k]);
                ++found;
            }
        }
    }
    // block totals of the counters
    unsigned fw = __reduce_add_sync(0xffffffffu, found);
    unsigned ew = __reduce_add_sync(0xffffffffu, evals);
    if ((tid & 31) == 0) {
        if (fw) atomicAdd(&ds->band_voxels, (unsigned long long)fw);
        if (ew) atomicAdd(&ds->splat_evals, (unsigned long long)ew);
    }
}

}  // namespace

void launch_prep(const float* tris12, long long T, const Lattice& L, SplatTri* sto, ParTri* pto,
                 unsigned* brick_count, unsigned* strip_count, DevState* ds, cudaStream_t st) {
    if (T <= 0) return;
    GBSDF_COUNT_LAUNCH();
    prep_kernel<<<(unsigned)((T + kPrepThreads - 1) / kPrepThreads), kPrepThreads, 0, st>>>(
        tris12, T, L, sto, pto, brick_count, strip_count, ds);
}

long long scan_tmp_elems(long long n) {
    long long total = 0;
    while (n > 1) {
        long long tiles = (n + kScanTile - 1) / kScanTile;
        total += 2 * tiles;
        n = tiles;
    }
    return total + 2;
}

void launch_exclusive_scan(const unsigned* in, unsigned long long* out, long long n, unsigned long long* tmp,
                           long long tmp_elems, cudaStream_t st) {
    (void)tmp_elems;
    if (n <= 0) return;
    scan_rec(in, false, out, n, tmp, st);
}

void launch_bin_fill(const SplatTri* stt, const ParTri* ptt, long long T, const Lattice& L,
                     const unsigned long long* brick_off, unsigned* brick_cur, unsigned* brick_list,
                     const unsigned long long* strip_off, unsigned* strip_cur, unsigned* strip_list,
                     cudaStream_t st, DevState* ds, unsigned long long cap_b, unsigned long long cap_s) {
    if (T <= 0) return;
    GBSDF_COUNT_LAUNCH();
    bin_fill_kernel<<<(unsigned)((T + kPrepThreads - 1) / kPrepThreads), kPrepThreads, 0, st>>>(
        stt, ptt, T, L, brick_off, brick_cur, brick_list, strip_off, strip_cur, strip_list, ds, cap_b, cap_s);
}

void launch_active_bricks(const unsigned* brick_count, long long nbricks, unsigned* active, DevState* ds,
                          cudaStream_t st, unsigned dense_cut) {
    GBSDF_COUNT_LAUNCH();
    active_bricks_kernel<<<(unsigned)((nbricks + 255) / 256), 256, 0, st>>>(brick_count, nbricks, active, ds,
                                                                            dense_cut);
}

void launch_fill(float* g, long long n, float value, cudaStream_t st) {
    long long n4 = n / 4;
    if (n4 > 0) {
        long long blocks = std::min<long long>((n4 + 255) / 256, 152LL * 32);
        GBSDF_COUNT_LAUNCH();
        fill_kernel<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<float4*>(g), n4, value);
    }
    if (n4 * 4 < n) { GBSDF_COUNT_LAUNCH(); fill_tail_kernel<<<1, 4, 0, st>>>(g, n4 * 4, n, value); }
}

namespace {
// One warp per sample: the lanes split the brick's triangle list, find the FP32 minimum
// (the splat's arithmetic), then evaluate in FP64 only the triangles whose FP32 squared
// distance lies within 0.1% (plus 1e-6 h^2) of it -- the FP64 minimum is among them.
constexpr int kBandErrWarps = 4;
__global__ void __launch_bounds__(kBandErrWarps * 32)
    band_error_kernel(const SplatTri* __restrict__ stt, const unsigned long long* __restrict__ boff,
                      const unsigned* __restrict__ bcount, const unsigned* __restrict__ blist, Lattice L,
                      const float* __restrict__ dist, DevState* ds) {
    const long long k = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= kBandErrSamples) return;
    // one voxel per stratum of N / kBandErrSamples, at a golden-ratio offset within it (an
    // offset common to all strata would put every sample in one x column when the stratum
    // is a multiple of the row length, as at 1024^3)
    const double off = (double)k * 0.6180339887498949 - floor((double)k * 0.6180339887498949);
    const long long v = (long long)(((double)k + off) * (double)L.N / (double)kBandErrSamples);
    if (v >= L.N) return;
    const float d = dist[v];
    if (!(d <= (float)kBandVoxels * L.h)) return;
    const int x = (int)(v % L.dims[0]);
    const long long r = v / L.dims[0];
    const int y = (int)(r % L.dims[1]), z = (int)(r / L.dims[1]);
    const long long b = ((long long)(z / kBrick) * L.nb[1] + y / kBrick) * L.nb[0] + x / kBrick;
    const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
    const unsigned long long e0 = boff[b], n = bcount[b];
    float m32 = 3.0e38f;
    for (unsigned long long e = lane; e < n; e += 32) {
        const float* t = stt[blist[e0 + e]].v;
        m32 = fminf(m32, ptd_sq(p, mk(t[0], t[1], t[2]), mk(t[3], t[4], t[5]), mk(t[6], t[7], t[8])));
    }
    for (int o = 16; o > 0; o >>= 1) m32 = fminf(m32, __shfl_xor_sync(0xffffffffu, m32, o));
    const float lim = m32 + m32 * 1e-3f + 1e-6f * L.h * L.h;
    double best = 1e300;
    for (unsigned long long e = lane; e < n; e += 32) {
        const float* t = stt[blist[e0 + e]].v;
        if (ptd_sq(p, mk(t[0], t[1], t[2]), mk(t[3], t[4], t[5]), mk(t[6], t[7], t[8])) <= lim)
            best = fmin(best, ptd_sq_f64(p.x, p.y, p.z, t));
    }
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (lane == 0) {
        const double err = fabs(sqrt(best) - (double)d) / (double)L.h;
        atomicMax(&ds->band_err_bits, (unsigned long long)__double_as_longlong(err));
        atomicAdd(&ds->band_err_n, 1ull);
    }
}
}  // namespace

void launch_band_error(const SplatTri* stt, const unsigned long long* brick_off, const unsigned* brick_count,
                       const unsigned* brick_list, const Lattice& L, const float* dist, DevState* ds, cudaStream_t st) {
    if (L.N <= 0) return;
    GBSDF_COUNT_LAUNCH();
    band_error_kernel<<<(unsigned)((kBandErrSamples + kBandErrWarps - 1) / kBandErrWarps), kBandErrWarps * 32, 0,
                        st>>>(stt, brick_off, brick_count, brick_list, L, dist, ds);
}

void launch_splat(const SplatTri* stt, const unsigned long long* brick_off, const unsigned* brick_count,
                  const unsigned* brick_list, const unsigned* active, long long n_active, long long n_dense,
                  const Lattice& L, float* dist, DevState* ds, cudaStream_t st) {
    const long long blocks = n_active < 0 ? L.nbricks : n_active;
    if (blocks > 0) {
        GBSDF_COUNT_LAUNCH();
        splat_kernel<<<(unsigned)blocks, kSplatThreads, 0, st>>>(stt, brick_off, brick_count, brick_list, active, L,
                                                                 dist, ds);
    }
    // dense bricks: known count, or read on the device with a grid-stride over at most 4096
    const long long dblocks = n_dense < 0 ? std::min<long long>(L.nbricks, 4096) : n_dense;
    if (dblocks > 0) {
        GBSDF_COUNT_LAUNCH();
        splat_dense_kernel<<<dim3((unsigned)dblocks, kDenseSlices), kDenseThreads, 0, st>>>(
            stt, brick_off, brick_count, brick_list, active, L, dist, ds);
        GBSDF_COUNT_LAUNCH();
        dense_count_kernel<<<(unsigned)std::min<long long>(dblocks, 1024), 256, 0, st>>>(active, L, dist, ds);
    }
}

}  // namespace gbsdf
