// k_eikonal.cu — FSM eikonal re-distancing [D], sentinel audit / clamp [D2]/[D3]
// and sign apply [F] of the mesh-to-SDF path.
//
// Reference: gpu_eikonal_fsm_sweep_kernel (cuda_rasterizer.cu:433-513) runs one thread
// per line walking the swept axis in place; the threads of axis-0 and axis-1 sweeps
// stride dim_x or 1 line apart, so their loads are uncoalesced. Lines of one sweep
// run concurrently and read each other's cells while they change.
//
// Here one sweep is a lockstep (Jacobi-across-lines) sweep: it reads a source copy
// of the grid and writes a destination copy, each line walked sequentially with the
// freshly updated upstream value carried in a register. Every line therefore sees
// its neighbour lines exactly as they were when the sweep began -- the deterministic
// model of the reference's launch of all lines at once -- and the result does not
// depend on scheduling. The source/destination pair alternates, so a sweep moves
// exactly 8 bytes per voxel through HBM (one 4-byte read, one 4-byte write).
//   * z and y sweeps: one thread per line, adjacent threads on adjacent x, so each
//     step of a warp is one 128-byte load and one 128-byte store;
//   * x sweeps: a CTA owns 16 x 8 lines, stages 34-voxel chunks of its lines plus the
//     one-line halo in shared memory with coalesced row loads, walks them, and
//     stores the chunk back with coalesced row stores.
// RULE 0 is the reference's update (godunov_ref), RULE 1 the corrected monotone one.
#include <algorithm>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

__device__ __forceinline__ void mark_changed(bool ch, int* flag) {
    unsigned b = __ballot_sync(__activemask(), ch);
    if (b && (threadIdx.x & 31) == __ffs(b) - 1) *flag = 1;
}

__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---- z and y sweeps: staged slab walk ----------------------------------------------
// A CTA owns a 32 (x) x 16 (rows) tile of lines, two lines per thread (rows r and
// r + 8); rows are y for a z sweep and z for a y sweep. The walk visits the lattice
// slices across the tile (z planes for a z sweep, y rows of every z for a y sweep).
// Each slice-tile with its one-cell halo (18 x 34 floats) is copied into a ring of 16
// shared-memory slots by cp.async, in batches of 4 slices issued two batches ahead,
// so the walk reads shared memory only, waits and synchronises once per 4 slices,
// and the DRAM latency of later slices overlaps the current batch. Out-of-lattice
// halo cells hold the far sentinel (the reference's boundary rule,
// cuda_rasterizer.cu:454-461). Each thread's copy addresses are computed once.
constexpr int kWX = 32, kWR = 16;            // tile: 32 x 16 lines
constexpr int kWThreads = 256;               // 2 lines per thread
constexpr int kWHX = kWX + 2, kWHR = kWR + 2;
constexpr int kWSlot = kWHX * kWHR;          // 612 floats per slice-tile
constexpr int kWB = 4;                       // slices per batch
constexpr int kWSlots = 16;                  // ring slots (4 batches)
constexpr int kWPer = (kWSlot + kWThreads - 1) / kWThreads;  // copies per thread per slice (3)
constexpr size_t kWSmem = (size_t)kWSlots * kWSlot * sizeof(float);

template <int AXIS, int RULE, int DIR>
__global__ void __launch_bounds__(kWThreads) sweep_walk_kernel(const float* __restrict__ src,
                                                               float* __restrict__ dst, Lattice L, int round,
                                                               DevState* ds) {
    if (ds->stop) return;
    extern __shared__ float ring[];
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const size_t plane = (size_t)dx * dy;
    const int n_walk = (AXIS == 2) ? dz : dy;
    const int n_rows = (AXIS == 2) ? dy : dz;
    const size_t step_stride = (AXIS == 2) ? plane : (size_t)dx;
    const size_t row_stride = (AXIS == 2) ? (size_t)dx : plane;
    const int tid = threadIdx.x, tx = tid & 31, tr = tid >> 5;
    const int x0 = blockIdx.x * kWX, r0 = blockIdx.y * kWR;
    const int x = x0 + tx;
    const int ra = r0 + tr, rb = r0 + tr + 8;
    const bool act_a = (x < dx) && (ra < n_rows), act_b = (x < dx) && (rb < n_rows);
    const float h = L.h;

    // this thread's copy descriptors (element e = tid + k * 256 of a slice-tile)
    long long goff[kWPer];
    unsigned inb = 0u;
#pragma unroll
    for (int k = 0; k < kWPer; ++k) {
        const int e = tid + k * kWThreads;
        const int rr = e / kWHX, cc = e - rr * kWHX;
        const int row = r0 - 1 + rr, col = x0 - 1 + cc;
        const bool ok = (e < kWSlot) && row >= 0 && row < n_rows && col >= 0 && col < dx;
        goff[k] = ok ? (long long)row * (long long)row_stride + col : 0;
        inb |= (ok ? 1u : 0u) << k;
        inb |= ((e < kWSlot) ? 1u : 0u) << (8 + k);
    }
    auto load_slice = [&](int s) {
        const int sl = (DIR > 0) ? s : (n_walk - 1 - s);
        float* slot = ring + (s & (kWSlots - 1)) * kWSlot;
        const float* base = src + (size_t)sl * step_stride;
#pragma unroll
        for (int k = 0; k < kWPer; ++k) {
            const int e = tid + k * kWThreads;
            if (inb & (1u << k)) cp_async4(slot + e, base + goff[k]);
            else if (inb & (1u << (8 + k))) slot[e] = kFarSentinel;
        }
    };
    auto load_batch = [&](int b) {
        for (int q = 0; q < kWB; ++q) {
            const int s = b * kWB + q;
            if (s < n_walk) load_slice(s);
        }
    };
    const int nbatches = (n_walk + kWB - 1) / kWB;
    load_batch(0);
    cp_async_commit();
    load_batch(1);
    cp_async_commit();
    const int ma = (tr + 1) * kWHX + (tx + 1), mb = ma + 8 * kWHX;
    float prev_a = kFarSentinel, prev_b = kFarSentinel;
    float cur_a = 0.0f, cur_b = 0.0f;  // value of the current slice, carried from the previous step
    bool ch = false;
    // output pointers of the two lines, advanced by one slice per step
    const long long sstep = (DIR > 0) ? (long long)step_stride : -(long long)step_stride;
    float* pa = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)ra * row_stride + x;
    float* pb = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)rb * row_stride + x;
#pragma unroll 1
    for (int b = 0; b < nbatches; ++b) {
        load_batch(b + 2);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        if (b == 0) {
            cur_a = ring[ma];
            cur_b = ring[mb];
        }
#pragma unroll
        for (int q = 0; q < kWB; ++q) {
            const int s = b * kWB + q;
            if (s >= n_walk) break;
            const float* cs = ring + (s & (kWSlots - 1)) * kWSlot;
            const float* ns = ring + ((s + 1) & (kWSlots - 1)) * kWSlot;
            const bool has_next = (s + 1 < n_walk);
            const float nxt_a = has_next ? ns[ma] : kFarSentinel;
            const float nxt_b = has_next ? ns[mb] : kFarSentinel;
            if (act_a) {
                const float ax = fminf(cs[ma - 1], cs[ma + 1]);
                const float ar = fminf(cs[ma - kWHX], cs[ma + kWHX]);
                const float al = fminf(prev_a, nxt_a);
                const float u = (AXIS == 2) ? godunov<RULE>(ax, ar, al, h) : godunov<RULE>(ax, al, ar, h);
                float out = cur_a;
                if (u < cur_a) {
                    out = u;
                    ch = true;
                }
                *pa = out;
                prev_a = out;
            }
            if (act_b) {
                const float ax = fminf(cs[mb - 1], cs[mb + 1]);
                const float ar = fminf(cs[mb - kWHX], cs[mb + kWHX]);
                const float al = fminf(prev_b, nxt_b);
                const float u = (AXIS == 2) ? godunov<RULE>(ax, ar, al, h) : godunov<RULE>(ax, al, ar, h);
                float out = cur_b;
                if (u < cur_b) {
                    out = u;
                    ch = true;
                }
                *pb = out;
                prev_b = out;
            }
            cur_a = nxt_a;
            cur_b = nxt_b;
            pa += sstep;
            pb += sstep;
        }
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- x sweeps: staged chunk walk ---------------------------------------------------
// A CTA owns 32 (y) x 8 (z) lines (one thread each) and walks x in chunks of 8 voxels.
// Each chunk of the 34 x 10 staged lines (tile plus one-line halo) goes into a ring of
// 4 shared-memory slots by cp.async two chunks ahead of the walk (8 consecutive floats
// of a line = one 32-byte sector). Lines are stored with an odd stride (9 floats) so
// the per-step reads of 32 lines hit 32 different banks. Results leave registers as
// two float4 stores per line and chunk.
constexpr int kXY = 32, kXZ = 8;                   // lines per CTA (threads)
constexpr int kXC = 8;                             // voxels per chunk
constexpr int kXStride = 9;                        // shared-memory floats per staged line
constexpr int kXHY = kXY + 2, kXHZ = kXZ + 2;
constexpr int kXLines = kXHY * kXHZ;               // 340 staged lines
constexpr int kXSlot = kXLines * kXStride;         // floats per ring slot
constexpr int kXS = 4, kXD = 2;                    // ring slots, prefetch distance
constexpr int kXThreads = kXY * kXZ;               // 256
constexpr size_t kXSmem = (size_t)kXS * kXSlot * sizeof(float);

template <int RULE, int DIR>
__global__ void __launch_bounds__(kXThreads) sweep_x_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                             Lattice L, int round, DevState* ds) {
    constexpr int dir = DIR;
    if (ds->stop) return;
    extern __shared__ float xring[];
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const float h = L.h;
    const size_t plane = (size_t)dx * dy;
    const int tid = threadIdx.x;
    const int ty = tid & 31, tz = tid >> 5;
    const int y0 = blockIdx.x * kXY, z0 = blockIdx.y * kXZ;
    const int y = y0 + ty, z = z0 + tz;
    const bool active = (y < dy) && (z < dz);
    const int nchunks = (dx + kXC - 1) / kXC;

    // copy descriptors: element e = tid + 256 k of a chunk is float j = e & 7 of staged
    // line e >> 3; 8 consecutive threads copy one line's 32-byte sector.
    constexpr int kXPer = (kXLines * kXC + kXThreads - 1) / kXThreads;  // 11
    const int jcopy = tid & 7;
    long long loff[kXPer];    // line start relative to the CTA's first (halo) line
    unsigned lok = 0u, lexist = 0u;
    const long long cta_base = (long long)(z0 - 1) * (long long)plane + (long long)(y0 - 1) * dx;
#pragma unroll
    for (int k = 0; k < kXPer; ++k) {
        const int ln = (tid >> 3) + 32 * k;
        const int hy = ln % kXHY, hz = ln / kXHY;
        const int yy = y0 - 1 + hy, zz = z0 - 1 + hz;
        const bool ex = ln < kXLines;
        const bool ok = ex && yy >= 0 && yy < dy && zz >= 0 && zz < dz;
        loff[k] = ok ? ((long long)zz * (long long)plane + (long long)yy * dx - cta_base) : 0;
        lok |= (ok ? 1u : 0u) << k;
        lexist |= (ex ? 1u : 0u) << k;
    }
    auto load_chunk = [&](int ci) {
        const int c = (dir > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        float* slot = xring + (ci % kXS) * kXSlot + jcopy;
        const bool xin = xc + jcopy < dx;
        const long long gb = cta_base + xc + jcopy;
#pragma unroll
        for (int k = 0; k < kXPer; ++k) {
            if (!(lexist & (1u << k))) continue;
            float* d = slot + ((tid >> 3) + 32 * k) * kXStride;
            if ((lok & (1u << k)) && xin) cp_async4(d, src + (gb + loff[k]));
            else *d = kFarSentinel;
        }
    };

#pragma unroll 1
    for (int d = 0; d < kXD; ++d) {
        if (d < nchunks) load_chunk(d);
        cp_async_commit();
    }
    const int me = (tz + 1) * kXHY + (ty + 1);
    const int n_ym = me - 1, n_yp = me + 1, n_zm = me - kXHY, n_zp = me + kXHY;
    float prev = kFarSentinel;
    bool ch = false;
#pragma unroll 1
    for (int ci = 0; ci < nchunks; ++ci) {
        if (ci + kXD < nchunks) load_chunk(ci + kXD);
        cp_async_commit();
        cp_async_wait<kXD - 1>();
        __syncthreads();
        const int c = (dir > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        if (active) {
            const float* cs = xring + (ci % kXS) * kXSlot;
            const float* ns = xring + ((ci + 1) % kXS) * kXSlot;  // next chunk in walk order
            float res[kXC];
            const bool fast = (xc + kXC <= dx) && (ci + 1 < nchunks);
            if (fast) {
#pragma unroll
                for (int jj = 0; jj < kXC; ++jj) {
                    const int j = (dir > 0) ? jj : (kXC - 1 - jj);
                    const float cur = cs[me * kXStride + j];
                    const float down = (dir > 0) ? ((j + 1 < kXC) ? cs[me * kXStride + j + 1] : ns[me * kXStride])
                                                 : ((j > 0) ? cs[me * kXStride + j - 1] : ns[me * kXStride + kXC - 1]);
                    const float ax = fminf(prev, down);
                    const float ay = fminf(cs[n_ym * kXStride + j], cs[n_yp * kXStride + j]);
                    const float az = fminf(cs[n_zm * kXStride + j], cs[n_zp * kXStride + j]);
                    const float u = godunov<RULE>(ax, ay, az, h);
                    const float out = (u < cur) ? u : cur;
                    ch |= (u < cur);
                    res[j] = out;
                    prev = out;
                }
            } else {
#pragma unroll
                for (int jj = 0; jj < kXC; ++jj) {
                    const int j = (dir > 0) ? jj : (kXC - 1 - jj);
                    const int x = xc + j;
                    res[j] = 0.0f;
                    if (x >= dx) continue;
                    const float cur = cs[me * kXStride + j];
                    float down;
                    if (dir > 0) down = (j + 1 < kXC) ? cs[me * kXStride + j + 1]
                                                     : ((ci + 1 < nchunks) ? ns[me * kXStride] : kFarSentinel);
                    else down = (j > 0) ? cs[me * kXStride + j - 1]
                                        : ((ci + 1 < nchunks) ? ns[me * kXStride + kXC - 1] : kFarSentinel);
                    const float ax = fminf(prev, down);
                    const float ay = fminf(cs[n_ym * kXStride + j], cs[n_yp * kXStride + j]);
                    const float az = fminf(cs[n_zm * kXStride + j], cs[n_zp * kXStride + j]);
                    const float u = godunov<RULE>(ax, ay, az, h);
                    const float out = (u < cur) ? u : cur;
                    ch |= (u < cur);
                    res[j] = out;
                    prev = out;
                }
            }
            float* drow = dst + (size_t)z * plane + (size_t)y * dx + xc;
            if (((dx & 3) == 0) && xc + kXC <= dx) {
                reinterpret_cast<float4*>(drow)[0] = make_float4(res[0], res[1], res[2], res[3]);
                reinterpret_cast<float4*>(drow)[1] = make_float4(res[4], res[5], res[6], res[7]);
            } else {
#pragma unroll
                for (int j = 0; j < kXC; ++j)
                    if (xc + j < dx) drow[j] = res[j];
            }
        }
    }
    mark_changed(ch, &ds->changed[round]);
}

__global__ void end_round_kernel(int slot, int round, int cap, DevState* ds) {
    if (ds->stop) return;
    ds->rounds = round + 1;
    if (!ds->changed[slot] || round + 1 >= cap) ds->stop = 1;
}

__global__ void audit_kernel(const float* __restrict__ g, long long n, unsigned long long* __restrict__ out) {
    long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) c += (g[i] >= 1e29f);
    c = __reduce_add_sync(0xffffffffu, (unsigned)c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}


// [D3] cuda_rasterizer.cu:544-556: leftover sentinels -> -band / +band by the signs of
// that moment (runs only when the audit found a residual). One CTA per 4 rows.
constexpr int kRowsPerCta = 4;
__global__ void clamp_kernel(float* __restrict__ g, const uint32_t* __restrict__ sbits, Lattice L, DevState* ds) {
    if (ds->far_residual == 0) return;
    const float bw = (float)kBandVoxels * L.h;
    const long long nrows = (long long)L.dims[1] * L.dims[2];
    for (int k = 0; k < kRowsPerCta; ++k) {
        const long long row = (long long)blockIdx.x * kRowsPerCta + k;
        if (row >= nrows) return;
        float* gr = g + row * L.dims[0];
        const uint32_t* sr = sbits + row * L.wx;
        for (int x = threadIdx.x; x < L.dims[0]; x += blockDim.x)
            if (gr[x] >= 1e29f) gr[x] = ((sr[x >> 5] >> (x & 31)) & 1u) ? -bw : bw;
    }
}

// [F] cuda_rasterizer.cu:650-661, applied only when the verify loop came back clean
// (on divergence the output stays untouched, cuda_rasterizer.cu:788-791). One CTA per
// 4 rows; float4 loads and stores when the row length allows.
// surf_tol (world units, 0 = off): voxels this close to the surface take the exact-
// arithmetic sign of a point on it (inside) -- the exact-signs modes.
__global__ void __launch_bounds__(256) apply_kernel(const float* __restrict__ g, const uint32_t* __restrict__ sbits,
                                                    Lattice L, float* __restrict__ out, const DevState* ds,
                                                    float surf_tol) {
    if (ds->verify_state != 1 || ds->abort_) return;
    const int dx = L.dims[0];
    const long long nrows = (long long)L.dims[1] * L.dims[2];
    const bool vec = (dx & 3) == 0;
    for (int k = 0; k < kRowsPerCta; ++k) {
        const long long row = (long long)blockIdx.x * kRowsPerCta + k;
        if (row >= nrows) return;
        const float* gr = g + row * dx;
        float* orow = out + row * dx;
        const uint32_t* sr = sbits + row * L.wx;
        if (vec) {
            for (int q = threadIdx.x; q < (dx >> 2); q += blockDim.x) {
                float4 d = reinterpret_cast<const float4*>(gr)[q];
                const int x = q << 2;
                const uint32_t w = sr[x >> 5] >> (x & 31);
                float v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float e = v[j];
                    if (e > 1e29f) e = 1e6f;
                    v[j] = (((w >> j) & 1u) || e <= surf_tol) ? -e : e;
                }
                reinterpret_cast<float4*>(orow)[q] = make_float4(v[0], v[1], v[2], v[3]);
            }
        } else {
            for (int x = threadIdx.x; x < dx; x += blockDim.x) {
                float e = gr[x];
                if (e > 1e29f) e = 1e6f;
                orow[x] = (((sr[x >> 5] >> (x & 31)) & 1u) || e <= surf_tol) ? -e : e;
            }
        }
    }
}

template <int RULE, int DIR>
void launch_sweep_t(int axis, int round, const float* src, float* dst, const Lattice& L, DevState* ds,
                    cudaStream_t st) {
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    GBSDF_COUNT_LAUNCH();
    if (axis == 2) {
        dim3 grid((dx + kWX - 1) / kWX, (dy + kWR - 1) / kWR);
        cudaFuncSetAttribute(sweep_walk_kernel<2, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kWSmem);
        sweep_walk_kernel<2, RULE, DIR><<<grid, kWThreads, kWSmem, st>>>(src, dst, L, round, ds);
    } else if (axis == 1) {
        dim3 grid((dx + kWX - 1) / kWX, (dz + kWR - 1) / kWR);
        cudaFuncSetAttribute(sweep_walk_kernel<1, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kWSmem);
        sweep_walk_kernel<1, RULE, DIR><<<grid, kWThreads, kWSmem, st>>>(src, dst, L, round, ds);
    } else {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        cudaFuncSetAttribute(sweep_x_kernel<RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kXSmem);
        sweep_x_kernel<RULE, DIR><<<grid, kXThreads, kXSmem, st>>>(src, dst, L, round, ds);
    }
}

}  // namespace

void launch_sweep(int rule, int axis, int dir, int round, const float* src, float* dst, const Lattice& L,
                  DevState* ds, cudaStream_t st) {
    if (rule == 0) {
        if (dir > 0) launch_sweep_t<0, 1>(axis, round, src, dst, L, ds, st);
        else launch_sweep_t<0, -1>(axis, round, src, dst, L, ds, st);
    } else {
        if (dir > 0) launch_sweep_t<1, 1>(axis, round, src, dst, L, ds, st);
        else launch_sweep_t<1, -1>(axis, round, src, dst, L, ds, st);
    }
}

void launch_end_round(int slot, int round, int cap, DevState* ds, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    end_round_kernel<<<1, 1, 0, st>>>(slot, round, cap, ds);
}

void launch_audit(const float* g, const Lattice& L, DevState* ds, cudaStream_t st) {
    long long blocks = std::min<long long>((L.N + 255) / 256, 152LL * 16);
    GBSDF_COUNT_LAUNCH();
    audit_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, L.N, &ds->far_residual);
}

void launch_clamp(float* g, const uint32_t* sbits, const Lattice& L, DevState* ds, cudaStream_t st) {
    long long blocks = ((long long)L.dims[1] * L.dims[2] + kRowsPerCta - 1) / kRowsPerCta;
    GBSDF_COUNT_LAUNCH();
    clamp_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, sbits, L, ds);
}

void launch_apply(const float* g, const uint32_t* sbits, const Lattice& L, float* out, const DevState* ds,
                  float surf_tol, cudaStream_t st) {
    long long blocks = ((long long)L.dims[1] * L.dims[2] + kRowsPerCta - 1) / kRowsPerCta;
    GBSDF_COUNT_LAUNCH();
    apply_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, sbits, L, out, ds, surf_tol);
}

}  // namespace gbsdf
