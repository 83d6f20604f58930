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
#include <vector>

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
    const size_t plane = (size_t)L.px * dy;
    const int n_walk = (AXIS == 2) ? dz : dy;
    const int n_rows = (AXIS == 2) ? dy : dz;
    const size_t step_stride = (AXIS == 2) ? plane : (size_t)L.px;
    const size_t row_stride = (AXIS == 2) ? (size_t)L.px : plane;
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
    const size_t plane = (size_t)L.px * dy;
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
    const long long cta_base = (long long)(z0 - 1) * (long long)plane + (long long)(y0 - 1) * L.px;
#pragma unroll
    for (int k = 0; k < kXPer; ++k) {
        const int ln = (tid >> 3) + 32 * k;
        const int hy = ln % kXHY, hz = ln / kXHY;
        const int yy = y0 - 1 + hy, zz = z0 - 1 + hz;
        const bool ex = ln < kXLines;
        const bool ok = ex && yy >= 0 && yy < dy && zz >= 0 && zz < dz;
        loff[k] = ok ? ((long long)zz * (long long)plane + (long long)yy * L.px - cta_base) : 0;
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
            float* drow = dst + (size_t)z * plane + (size_t)y * L.px + xc;
            if (((L.px & 3) == 0) && xc + kXC <= dx) {
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

// ---- x sweeps, TMA-staged ------------------------------------------------------------
// Same lines per CTA (32 y x 8 z), chunks (8 voxels) and ring as sweep_x_kernel, but each
// chunk of the 34 x 10 staged lines is ONE cp.async.bulk.tensor copy issued by one thread,
// completing on an mbarrier: no per-thread copy instructions. The tile lands with the
// 32-byte swizzle (the two 16-byte halves of a 32-byte line are swapped on every other
// group of four lines), so each thread reads its own line and its four neighbour lines
// as 16-byte vectors with no bank conflicts (8 consecutive lines of a quarter-warp hit 8
// distinct 16-byte bank groups). Out-of-lattice cells arrive as NaN; the neighbour-pair
// minimum with the far sentinel turns them into it (fminf drops a NaN operand), which is
// the reference's boundary rule (cuda_rasterizer.cu:454-461) bit for bit.
// Every wait on a tile is bounded: on a timeout the CTA waits (bounded) for its copies in
// flight, counts the event in DevState::wait_timeouts and returns.
constexpr int kTBox = kXC * kXHY * kXHZ;            // floats per staged tile (2720)
constexpr int kTSlotBytes = 11264;                  // tile bytes rounded up to 1 KB
constexpr int kTS = 4, kTD = 2;                     // ring slots, prefetch distance
constexpr size_t kTSmem = (size_t)kTS * kTSlotBytes + 64 + 1024;
// A tile wait polls the barrier at most kWaitPolls times; each poll suspends the waiting
// thread until the phase completes or kWaitSuspendNs pass, so a wait ends within about
// 2.6 s even when its copy never lands, and a thread whose tile is late does not spin.
constexpr int kWaitPolls = 1 << 17;
constexpr unsigned kWaitSuspendNs = 20000;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kWaitSuspendNs)
        : "memory");
    return ok != 0;
}
// `polls` bounds the wait (a build's DevState::wait_polls, wait_poll_limit below); the
// drains that let a leaving CTA's copies land always use the full kWaitPolls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int polls = kWaitPolls) {
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// The poll limit of a build's tile waits: kWaitPolls by default (DevState::wait_polls 0), a
// caller's limit when positive, none at all when negative (every wait gives up at once --
// the failure path's test).
__device__ __forceinline__ int wait_poll_limit(const DevState* ds) {
    const int w = ds->wait_polls;
    return w == 0 ? kWaitPolls : (w > 0 ? w : 0);
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// float offset of element j (0..7) of staged line r in a 32-byte-swizzled tile
__device__ __forceinline__ int tsw(int r, int j) { return r * 8 + ((((j >> 2) ^ (r >> 2)) & 1) << 2) + (j & 3); }
// 16-byte half c (0, 1) of staged line r
__device__ __forceinline__ float4 tvec(const float* tile, int r, int c) {
    return reinterpret_cast<const float4*>(tile)[r * 2 + ((c ^ (r >> 2)) & 1)];
}
// The first 1 KB-aligned byte of a dynamic shared-memory array (TMA tiles and their
// swizzle want 1 KB alignment of the shared-window address). Offsetting the array's own
// pointer, rather than rounding an integer, keeps the shared address space visible to the
// compiler, so tile reads are shared-memory loads and not generic ones.
__device__ __forceinline__ unsigned char* align1k(unsigned char* p) {
    return p + ((1024u - (smem_u32(p) & 1023u)) & 1023u);
}

template <int RULE, int DIR>
__global__ void __launch_bounds__(kXThreads) sweep_x_tma_kernel(const __grid_constant__ CUtensorMap tm,
                                                                 float* __restrict__ dst, Lattice L, int round,
                                                                 DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(tsm + kTS * kTSlotBytes);
    __shared__ int s_ok;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const float h = L.h;
    const size_t plane = (size_t)L.px * dy;
    const int tid = threadIdx.x, ty = tid & 31, tz = tid >> 5;
    const int y0 = blockIdx.x * kXY, z0 = blockIdx.y * kXZ;
    const int y = y0 + ty, z = z0 + tz;
    const bool active = (y < dy) && (z < dz);
    const int nchunks = (dx + kXC - 1) / kXC;
    auto issue = [&](int ci) {
        const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
        const int s = ci % kTS;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_expect_tx(&bars[s], kTBox * 4);
        tma_load_3d(tsm + s * kTSlotBytes, &tm, c * kXC, y0 - 1, z0 - 1, &bars[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < kTS; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_ok = 1;
        for (int d = 0; d < kTD && d < nchunks; ++d) issue(d);
    }
    const int rme = (tz + 1) * kXHY + (ty + 1);
    const int rym = rme - 1, ryp = rme + 1, rzm = rme - kXHY, rzp = rme + kXHY;
    float prev = kFarSentinel;
    bool ch = false;
#pragma unroll 1
    for (int ci = 0; ci < nchunks; ++ci) {
        __syncthreads();  // every thread is done with chunk ci - 1, so slot (ci + kTD) % kTS is free
        if (tid == 0) {
            if (ci + kTD < nchunks) issue(ci + kTD);
            bool ok = mbar_wait(&bars[ci % kTS], (ci / kTS) & 1, polls);
            if (ok && ci + 1 < nchunks) ok = mbar_wait(&bars[(ci + 1) % kTS], ((ci + 1) / kTS) & 1, polls);
            if (!ok) {
                // let the copies still in flight land before the CTA's shared memory goes
                for (int k = ci; k < min(nchunks, ci + kTD + 1); ++k) mbar_wait(&bars[k % kTS], (k / kTS) & 1);
                atomicAdd(&ds->wait_timeouts, 1ull);
                s_ok = 0;
            }
        }
        __syncthreads();
        if (!s_ok) return;
        const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        if (!active) continue;
        const float* tile = reinterpret_cast<const float*>(tsm + (ci % kTS) * kTSlotBytes);
        const float* ntile = reinterpret_cast<const float*>(tsm + ((ci + 1) % kTS) * kTSlotBytes);
        float res[kXC];
        if (xc + kXC <= dx && ci + 1 < nchunks) {
            float cur[kXC], ay[kXC], az[kXC];
            {
                const float4 m0 = tvec(tile, rme, 0), m1 = tvec(tile, rme, 1);
                cur[0] = m0.x; cur[1] = m0.y; cur[2] = m0.z; cur[3] = m0.w;
                cur[4] = m1.x; cur[5] = m1.y; cur[6] = m1.z; cur[7] = m1.w;
            }
#pragma unroll
            for (int hv = 0; hv < 2; ++hv) {
                const float4 a = tvec(tile, rym, hv), b = tvec(tile, ryp, hv);
                const float4 p = tvec(tile, rzm, hv), q = tvec(tile, rzp, hv);
                ay[4 * hv + 0] = fminf(fminf(a.x, b.x), kFarSentinel);
                ay[4 * hv + 1] = fminf(fminf(a.y, b.y), kFarSentinel);
                ay[4 * hv + 2] = fminf(fminf(a.z, b.z), kFarSentinel);
                ay[4 * hv + 3] = fminf(fminf(a.w, b.w), kFarSentinel);
                az[4 * hv + 0] = fminf(fminf(p.x, q.x), kFarSentinel);
                az[4 * hv + 1] = fminf(fminf(p.y, q.y), kFarSentinel);
                az[4 * hv + 2] = fminf(fminf(p.z, q.z), kFarSentinel);
                az[4 * hv + 3] = fminf(fminf(p.w, q.w), kFarSentinel);
            }
            // the first voxel of the next chunk in walk order
            const float nxt = (DIR > 0) ? ntile[tsw(rme, 0)] : ntile[tsw(rme, kXC - 1)];
#pragma unroll
            for (int jj = 0; jj < kXC; ++jj) {
                const int j = (DIR > 0) ? jj : (kXC - 1 - jj);
                const float down = (DIR > 0) ? ((j + 1 < kXC) ? cur[j + 1] : nxt) : ((j > 0) ? cur[j - 1] : nxt);
                const float u = godunov<RULE>(fminf(prev, down), ay[j], az[j], h);
                const float out = (u < cur[j]) ? u : cur[j];
                ch |= (u < cur[j]);
                res[j] = out;
                prev = out;
            }
        } else {
#pragma unroll
            for (int jj = 0; jj < kXC; ++jj) {
                const int j = (DIR > 0) ? jj : (kXC - 1 - jj);
                res[j] = 0.0f;
                if (xc + j >= dx) continue;
                const float cur = tile[tsw(rme, j)];
                float down;
                if (DIR > 0) down = (j + 1 < kXC) ? tile[tsw(rme, j + 1)]
                                                  : ((ci + 1 < nchunks) ? ntile[tsw(rme, 0)] : kFarSentinel);
                else down = (j > 0) ? tile[tsw(rme, j - 1)]
                                    : ((ci + 1 < nchunks) ? ntile[tsw(rme, kXC - 1)] : kFarSentinel);
                const float ayj = fminf(fminf(tile[tsw(rym, j)], tile[tsw(ryp, j)]), kFarSentinel);
                const float azj = fminf(fminf(tile[tsw(rzm, j)], tile[tsw(rzp, j)]), kFarSentinel);
                const float u = godunov<RULE>(fminf(prev, down), ayj, azj, h);
                const float out = (u < cur) ? u : cur;
                ch |= (u < cur);
                res[j] = out;
                prev = out;
            }
        }
        float* drow = dst + (size_t)z * plane + (size_t)y * L.px + xc;
        if (xc + kXC <= dx) {
            reinterpret_cast<float4*>(drow)[0] = make_float4(res[0], res[1], res[2], res[3]);
            reinterpret_cast<float4*>(drow)[1] = make_float4(res[4], res[5], res[6], res[7]);
        } else {
#pragma unroll
            for (int j = 0; j < kXC; ++j)
                if (xc + j < dx) drow[j] = res[j];
        }
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- x sweeps, TMA-staged, warp-specialised pipeline ---------------------------------
// The tiles, swizzle and per-line arithmetic of sweep_x_tma_kernel, with the ring run as
// a producer / consumer pipeline on mbarriers instead of CTA-wide barriers: warp 8 issues
// the bulk copies (waiting for a slot's "empty" barrier, 8 warp arrivals), the 8 consumer
// warps each wait for the "full" barriers of the chunks they read and release a slot when
// their last read of it is done. Warps drift up to the ring depth apart, so the serial
// chains of different warps overlap instead of meeting at a barrier every chunk. All
// waits are bounded; a warp that gives up counts the event and leaves, and the producer
// lets its copies in flight land before it leaves.
constexpr int kPS = 4;                               // ring slots
constexpr int kPThreads = kXThreads + 32;            // 8 consumer warps + 1 producer warp
constexpr size_t kPSmem = (size_t)kPS * kTSlotBytes + 128 + 1024;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// NB: the reference's update without branches, RULE 0 at voxel sizes with pair_sqrt_ok
// (1: godunov_ref_nb; 2: godunov_ref_nbp, its 2D and 3D arithmetic paired on packed FP32
// lanes, 57-59 instructions per voxel against 66), identical results.
template <int RULE, int DIR, int NB = 0>
__global__ void __launch_bounds__(kPThreads) sweep_x_pipe_kernel(const __grid_constant__ CUtensorMap tm,
                                                                  float* __restrict__ dst, Lattice L, int round,
                                                                  DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kPS * kTSlotBytes);
    uint64_t* empty = full + kPS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const float h = L.h;
    const float m2h = -2.0f * h, na3 = -(3.0f * h * h);
    const GodunovOneConsts gc = godunov_one_consts(h);
    const size_t plane = (size_t)L.px * dy;
    const int tid = threadIdx.x;
    const int y0 = blockIdx.x * kXY, z0 = blockIdx.y * kXZ;
    const int nchunks = (dx + kXC - 1) / kXC;
    if (tid == 0) {
        for (int s = 0; s < kPS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kXThreads / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();  // the only CTA-wide barrier: the ring's barriers are initialised
    if (tid >= kXThreads) {
        // producer warp: one lane issues every chunk's copy
        if (tid != kXThreads) return;
        int ci = 0;
        for (; ci < nchunks; ++ci) {
            const int s = ci % kPS;
            if (ci >= kPS && !mbar_wait(&empty[s], ((ci / kPS) - 1) & 1, polls)) break;
            const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kTBox * 4);
            tma_load_3d(tsm + s * kTSlotBytes, &tm, c * kXC, y0 - 1, z0 - 1, &full[s]);
        }
        // let every copy still in flight land before the producer leaves (consumers that gave
        // up have left already); a break means the consumers stopped releasing slots
        for (int k = max(0, ci - kPS); k < ci; ++k) mbar_wait(&full[k % kPS], (k / kPS) & 1);
        if (ci < nchunks) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int ty = tid & 31, tz = tid >> 5;
    const int y = y0 + ty, z = z0 + tz;
    const bool active = (y < dy) && (z < dz);
    const int rme = (tz + 1) * kXHY + (ty + 1);
    const int rym = rme - 1, ryp = rme + 1, rzm = rme - kXHY, rzp = rme + kXHY;
    float prev = kFarSentinel;
    bool ch = false;
#pragma unroll 1
    for (int ci = 0; ci < nchunks; ++ci) {
        bool ok = mbar_wait(&full[ci % kPS], (ci / kPS) & 1, polls);
        if (ok && ci + 1 < nchunks) ok = mbar_wait(&full[(ci + 1) % kPS], ((ci + 1) / kPS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if (ty == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        if (active) {
            const float* tile = reinterpret_cast<const float*>(tsm + (ci % kPS) * kTSlotBytes);
            const float* ntile = reinterpret_cast<const float*>(tsm + ((ci + 1) % kPS) * kTSlotBytes);
            float res[kXC];
            if (xc + kXC <= dx && ci + 1 < nchunks) {
                float cur[kXC], ay[kXC], az[kXC];
                {
                    const float4 m0 = tvec(tile, rme, 0), m1 = tvec(tile, rme, 1);
                    cur[0] = m0.x; cur[1] = m0.y; cur[2] = m0.z; cur[3] = m0.w;
                    cur[4] = m1.x; cur[5] = m1.y; cur[6] = m1.z; cur[7] = m1.w;
                }
#pragma unroll
                for (int hv = 0; hv < 2; ++hv) {
                    const float4 a = tvec(tile, rym, hv), b = tvec(tile, ryp, hv);
                    const float4 p = tvec(tile, rzm, hv), q = tvec(tile, rzp, hv);
                    ay[4 * hv + 0] = min3f(a.x, b.x, kFarSentinel);
                    ay[4 * hv + 1] = min3f(a.y, b.y, kFarSentinel);
                    ay[4 * hv + 2] = min3f(a.z, b.z, kFarSentinel);
                    ay[4 * hv + 3] = min3f(a.w, b.w, kFarSentinel);
                    az[4 * hv + 0] = min3f(p.x, q.x, kFarSentinel);
                    az[4 * hv + 1] = min3f(p.y, q.y, kFarSentinel);
                    az[4 * hv + 2] = min3f(p.z, q.z, kFarSentinel);
                    az[4 * hv + 3] = min3f(p.w, q.w, kFarSentinel);
                }
                const float nxt = (DIR > 0) ? ntile[tsw(rme, 0)] : ntile[tsw(rme, kXC - 1)];
#pragma unroll
                for (int jj = 0; jj < kXC; ++jj) {
                    const int j = (DIR > 0) ? jj : (kXC - 1 - jj);
                    const float down = (DIR > 0) ? ((j + 1 < kXC) ? cur[j + 1] : nxt) : ((j > 0) ? cur[j - 1] : nxt);
                    float u;
                    if constexpr (NB == 2) u = godunov_ref_nbp(fminf(prev, down), ay[j], az[j], gc);
                    else if constexpr (NB == 1) u = godunov_ref_nb(fminf(prev, down), ay[j], az[j], h, m2h, na3);
                    else u = godunov<RULE>(fminf(prev, down), ay[j], az[j], h);
                    const float out = (u < cur[j]) ? u : cur[j];
                    ch |= (u < cur[j]);
                    res[j] = out;
                    prev = out;
                }
            } else {
#pragma unroll
                for (int jj = 0; jj < kXC; ++jj) {
                    const int j = (DIR > 0) ? jj : (kXC - 1 - jj);
                    res[j] = 0.0f;
                    if (xc + j >= dx) continue;
                    const float cur = tile[tsw(rme, j)];
                    float down;
                    if (DIR > 0) down = (j + 1 < kXC) ? tile[tsw(rme, j + 1)]
                                                      : ((ci + 1 < nchunks) ? ntile[tsw(rme, 0)] : kFarSentinel);
                    else down = (j > 0) ? tile[tsw(rme, j - 1)]
                                        : ((ci + 1 < nchunks) ? ntile[tsw(rme, kXC - 1)] : kFarSentinel);
                    const float ayj = fminf(fminf(tile[tsw(rym, j)], tile[tsw(ryp, j)]), kFarSentinel);
                    const float azj = fminf(fminf(tile[tsw(rzm, j)], tile[tsw(rzp, j)]), kFarSentinel);
                    const float u = godunov<RULE>(fminf(prev, down), ayj, azj, h);
                    const float out = (u < cur) ? u : cur;
                    ch |= (u < cur);
                    res[j] = out;
                    prev = out;
                }
            }
            float* drow = dst + (size_t)z * plane + (size_t)y * L.px + xc;
            if (xc + kXC <= dx) {
                reinterpret_cast<float4*>(drow)[0] = make_float4(res[0], res[1], res[2], res[3]);
                reinterpret_cast<float4*>(drow)[1] = make_float4(res[4], res[5], res[6], res[7]);
            } else {
#pragma unroll
                for (int j = 0; j < kXC; ++j)
                    if (xc + j < dx) drow[j] = res[j];
            }
        }
        // this warp's last read of chunk ci's slot is done (it was also chunk ci-1's "next")
        __syncwarp();
        if (ty == 0) mbar_arrive(&empty[ci % kPS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- x sweeps, TMA pipeline, two lines per thread updated in packed pairs ------------
// sweep_x_pipe_kernel's tiles, ring and barriers with 4 consumer warps: the thread of
// lane ty in warp w walks the lines (y0 + ty, z0 + w) and (y0 + ty, z0 + w + 4), and the
// two serial chains advance together, their reference updates computed by
// godunov_ref_pair on packed FP32 pairs (same roundings, half the arithmetic issue
// slots). The neighbour minima skip the far-sentinel clamp, which a lattice with at least
// two voxels along y and z never needs (an out-of-lattice NaN always meets an in-lattice
// partner); the launcher falls back to sweep_x_pipe_kernel elsewhere.
constexpr int kP2Consumers = kXThreads / 2;              // 4 consumer warps
constexpr int kP2Threads = kP2Consumers + 32;

template <int DIR>
__global__ void __launch_bounds__(kP2Threads, 4) sweep_x_pipe2_kernel(const __grid_constant__ CUtensorMap tm,
                                                                   float* __restrict__ dst, Lattice L, int round,
                                                                   DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kPS * kTSlotBytes);
    uint64_t* empty = full + kPS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const size_t plane = (size_t)L.px * dy;
    const int tid = threadIdx.x;
    const int y0 = blockIdx.x * kXY, z0 = blockIdx.y * kXZ;
    const int nchunks = (dx + kXC - 1) / kXC;
    if (tid == 0) {
        for (int s = 0; s < kPS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kP2Consumers / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();  // the only CTA-wide barrier: the ring's barriers are initialised
    if (tid >= kP2Consumers) {
        if (tid != kP2Consumers) return;
        int ci = 0;
        for (; ci < nchunks; ++ci) {
            const int s = ci % kPS;
            if (ci >= kPS && !mbar_wait(&empty[s], ((ci / kPS) - 1) & 1, polls)) break;
            const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kTBox * 4);
            tma_load_3d(tsm + s * kTSlotBytes, &tm, c * kXC, y0 - 1, z0 - 1, &full[s]);
        }
        // let every copy still in flight land before the producer leaves (consumers that gave
        // up have left already); a break means the consumers stopped releasing slots
        for (int k = max(0, ci - kPS); k < ci; ++k) mbar_wait(&full[k % kPS], (k / kPS) & 1);
        if (ci < nchunks) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int ty = tid & 31, tz = tid >> 5;
    const int y = y0 + ty;
    const int za = z0 + tz, zb = z0 + tz + 4;
    const bool act_a = (y < dy) && (za < dz), act_b = (y < dy) && (zb < dz);
    const int rma = (tz + 1) * kXHY + (ty + 1), rmb = rma + 4 * kXHY;
    const GodunovPairConsts gc = godunov_pair_consts(L.h);
    const float h = L.h;
    float preva = kFarSentinel, prevb = kFarSentinel;
    bool ch = false;
#pragma unroll 1
    for (int ci = 0; ci < nchunks; ++ci) {
        bool ok = mbar_wait(&full[ci % kPS], (ci / kPS) & 1, polls);
        if (ok && ci + 1 < nchunks) ok = mbar_wait(&full[(ci + 1) % kPS], ((ci + 1) / kPS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if (ty == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        const float* tile = reinterpret_cast<const float*>(tsm + (ci % kPS) * kTSlotBytes);
        const float* ntile = reinterpret_cast<const float*>(tsm + ((ci + 1) % kPS) * kTSlotBytes);
        if (act_a && xc + kXC <= dx && ci + 1 < nchunks) {
            // both lines' chunks are whole (line b may be outside the lattice: it then
            // reads the NaN fill and its results are not stored). The chunk is walked in
            // two 4-voxel halves, so only one half's operands are live at a time.
            float* da = dst + (size_t)za * plane + (size_t)y * L.px + xc;
            float* db = dst + (size_t)zb * plane + (size_t)y * L.px + xc;
            const float nxta = (DIR > 0) ? ntile[tsw(rma, 0)] : ntile[tsw(rma, kXC - 1)];
            const float nxtb = (DIR > 0) ? ntile[tsw(rmb, 0)] : ntile[tsw(rmb, kXC - 1)];
            float4 ma = tvec(tile, rma, (DIR > 0) ? 0 : 1), mb = tvec(tile, rmb, (DIR > 0) ? 0 : 1);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int hv = (DIR > 0) ? k : 1 - k;
                const float cura[4] = {ma.x, ma.y, ma.z, ma.w}, curb[4] = {mb.x, mb.y, mb.z, mb.w};
                float enda, endb;  // the other half's first cell in walk order, or the next chunk's
                if (k == 0) {
                    const float4 na = tvec(tile, rma, 1 - hv), nb = tvec(tile, rmb, 1 - hv);
                    enda = (DIR > 0) ? na.x : na.w;
                    endb = (DIR > 0) ? nb.x : nb.w;
                    ma = na;
                    mb = nb;
                } else {
                    enda = nxta;
                    endb = nxtb;
                }
                const float4 a = tvec(tile, rma - 1, hv), b = tvec(tile, rma + 1, hv);
                const float4 p = tvec(tile, rma - kXHY, hv), q = tvec(tile, rma + kXHY, hv);
                const float4 a2 = tvec(tile, rmb - 1, hv), b2 = tvec(tile, rmb + 1, hv);
                const float4 p2 = tvec(tile, rmb - kXHY, hv), q2 = tvec(tile, rmb + kXHY, hv);
                const float aya[4] = {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w)};
                const float aza[4] = {fminf(p.x, q.x), fminf(p.y, q.y), fminf(p.z, q.z), fminf(p.w, q.w)};
                const float ayb[4] = {fminf(a2.x, b2.x), fminf(a2.y, b2.y), fminf(a2.z, b2.z), fminf(a2.w, b2.w)};
                const float azb[4] = {fminf(p2.x, q2.x), fminf(p2.y, q2.y), fminf(p2.z, q2.z), fminf(p2.w, q2.w)};
                float resa[4], resb[4];
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const int j = (DIR > 0) ? jj : (3 - jj);
                    const float downa = (DIR > 0) ? ((j + 1 < 4) ? cura[j + 1] : enda) : ((j > 0) ? cura[j - 1] : enda);
                    const float downb = (DIR > 0) ? ((j + 1 < 4) ? curb[j + 1] : endb) : ((j > 0) ? curb[j - 1] : endb);
                    float ua, ub;
                    godunov_ref_pair(fminf(preva, downa), aya[j], aza[j], fminf(prevb, downb), ayb[j], azb[j], gc, ua,
                                     ub);
                    const bool la = ua < cura[j], lb = act_b && (ub < curb[j]);
                    resa[j] = la ? ua : cura[j];
                    resb[j] = lb ? ub : curb[j];
                    ch |= la | lb;
                    preva = resa[j];
                    prevb = resb[j];
                }
                reinterpret_cast<float4*>(da)[hv] = make_float4(resa[0], resa[1], resa[2], resa[3]);
                if (act_b) reinterpret_cast<float4*>(db)[hv] = make_float4(resb[0], resb[1], resb[2], resb[3]);
            }
        } else {
            // a partial or the last chunk: each line on its own with the scalar update
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const bool act = side ? act_b : act_a;
                if (!act) continue;
                const int rme = side ? rmb : rma;
                const int z = side ? zb : za;
                float prev = side ? prevb : preva;
                float res[kXC];
#pragma unroll
                for (int jj = 0; jj < kXC; ++jj) {
                    const int j = (DIR > 0) ? jj : (kXC - 1 - jj);
                    res[j] = 0.0f;
                    if (xc + j >= dx) continue;
                    const float cur = tile[tsw(rme, j)];
                    float down;
                    if (DIR > 0) down = (j + 1 < kXC) ? tile[tsw(rme, j + 1)]
                                                      : ((ci + 1 < nchunks) ? ntile[tsw(rme, 0)] : kFarSentinel);
                    else down = (j > 0) ? tile[tsw(rme, j - 1)]
                                        : ((ci + 1 < nchunks) ? ntile[tsw(rme, kXC - 1)] : kFarSentinel);
                    const float ayj = fminf(tile[tsw(rme - 1, j)], tile[tsw(rme + 1, j)]);
                    const float azj = fminf(tile[tsw(rme - kXHY, j)], tile[tsw(rme + kXHY, j)]);
                    const float u = godunov_ref(fminf(prev, down), ayj, azj, h);
                    const float out = (u < cur) ? u : cur;
                    ch |= (u < cur);
                    res[j] = out;
                    prev = out;
                }
                float* drow = dst + (size_t)z * plane + (size_t)y * L.px + xc;
                if (xc + kXC <= dx) {
                    reinterpret_cast<float4*>(drow)[0] = make_float4(res[0], res[1], res[2], res[3]);
                    reinterpret_cast<float4*>(drow)[1] = make_float4(res[4], res[5], res[6], res[7]);
                } else {
#pragma unroll
                    for (int j = 0; j < kXC; ++j)
                        if (xc + j < dx) drow[j] = res[j];
                }
                if (side) prevb = prev;
                else preva = prev;
            }
        }
        // this warp's last read of chunk ci's slot is done (it was also chunk ci-1's "next")
        __syncwarp();
        if (ty == 0) mbar_arrive(&empty[ci % kPS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- x sweeps, wide TMA tiles ----------------------------------------------------------
// sweep_x_pipe_kernel's lines, warps and per-line arithmetic with 16-voxel chunks staged as
// 20 (x) x 34 (y) x 10 (z) boxes: 80-byte rows, fewer and longer rows per copy than the
// 32-byte rows of the 8-voxel chunks. No swizzle is needed: at a row pitch of 20 words, 8
// lanes' 16-byte loads of 8 consecutive rows fall in 32 distinct banks. A box starts at
// x = 16c (DIR > 0: its last 4 columns are the next chunk's first) or 16c - 4 (DIR < 0: its
// first 4 columns are the previous chunk's last), 16-byte aligned either way (a negative
// start reads the out-of-lattice fill), so a chunk's downstream neighbour arrives with it
// and each chunk waits for one copy. A 2-slot ring; every wait bounded as in the pipeline.
constexpr int kXW = 16;                                       // voxels per chunk
constexpr int kXWB = kXW + 4;                                 // box columns
constexpr int kXWS = 2;                                       // ring slots
constexpr int kXWBox = kXWB * kXHY * kXHZ;                    // floats per box (6800)
constexpr int kXWSlotBytes = (kXWBox * 4 + 1023) / 1024 * 1024;
constexpr size_t kXWSmem = (size_t)kXWS * kXWSlotBytes + 64 + 1024;

template <int RULE, int DIR, bool NB>
__global__ void __launch_bounds__(kPThreads) sweep_x_wide_kernel(const __grid_constant__ CUtensorMap tm,
                                                                  float* __restrict__ dst, Lattice L, int round,
                                                                  DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kXWS * kXWSlotBytes);
    uint64_t* empty = full + kXWS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const float h = L.h;
    const float m2h = -2.0f * h, na3 = -(3.0f * h * h);
    const size_t plane = (size_t)L.px * dy;
    const int tid = threadIdx.x;
    const int y0 = blockIdx.x * kXY, z0 = blockIdx.y * kXZ;
    const int nchunks = (dx + kXW - 1) / kXW;
    if (tid == 0) {
        for (int s = 0; s < kXWS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kXThreads / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();  // the only CTA-wide barrier: the ring's barriers are initialised
    if (tid >= kXThreads) {
        if (tid != kXThreads) return;
        int ci = 0;
        for (; ci < nchunks; ++ci) {
            const int s = ci % kXWS;
            if (ci >= kXWS && !mbar_wait(&empty[s], ((ci / kXWS) - 1) & 1, polls)) break;
            const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kXWBox * 4);
            tma_load_3d(tsm + s * kXWSlotBytes, &tm, (DIR > 0) ? c * kXW : c * kXW - 4, y0 - 1, z0 - 1, &full[s]);
        }
        for (int k = max(0, ci - kXWS); k < ci; ++k) mbar_wait(&full[k % kXWS], (k / kXWS) & 1);
        if (ci < nchunks) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int ty = tid & 31, tz = tid >> 5;
    const int y = y0 + ty, z = z0 + tz;
    const bool active = (y < dy) && (z < dz);
    const int rme = (tz + 1) * kXHY + (ty + 1);
    const int cb = (DIR > 0) ? 0 : 4;  // tile column of the chunk's first voxel
    float prev = kFarSentinel;
    bool ch = false;
#pragma unroll 1
    for (int ci = 0; ci < nchunks; ++ci) {
        const bool ok = mbar_wait(&full[ci % kXWS], (ci / kXWS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if (ty == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        const int c = (DIR > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXW;
        if (active) {
            const float* tile = reinterpret_cast<const float*>(tsm + (ci % kXWS) * kXWSlotBytes);
            const float* me = tile + rme * kXWB + cb;
            const float* yl = tile + (rme - 1) * kXWB + cb;
            const float* yh = tile + (rme + 1) * kXWB + cb;
            const float* zl = tile + (rme - kXHY) * kXWB + cb;
            const float* zh = tile + (rme + kXHY) * kXWB + cb;
            float* drow = dst + (size_t)z * plane + (size_t)y * L.px + xc;
            if (xc + kXW <= dx) {
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const int q = (DIR > 0) ? qq : 3 - qq;
                    const float4 m = *reinterpret_cast<const float4*>(me + 4 * q);
                    const float4 a = *reinterpret_cast<const float4*>(yl + 4 * q);
                    const float4 b = *reinterpret_cast<const float4*>(yh + 4 * q);
                    const float4 p = *reinterpret_cast<const float4*>(zl + 4 * q);
                    const float4 r = *reinterpret_cast<const float4*>(zh + 4 * q);
                    const float cur[4] = {m.x, m.y, m.z, m.w};
                    const float ay[4] = {min3f(a.x, b.x, kFarSentinel), min3f(a.y, b.y, kFarSentinel),
                                         min3f(a.z, b.z, kFarSentinel), min3f(a.w, b.w, kFarSentinel)};
                    const float az[4] = {min3f(p.x, r.x, kFarSentinel), min3f(p.y, r.y, kFarSentinel),
                                         min3f(p.z, r.z, kFarSentinel), min3f(p.w, r.w, kFarSentinel)};
                    // the quad's downstream neighbour beyond its last cell in walk order
                    const int xe = (DIR > 0) ? xc + 4 * q + 4 : xc + 4 * q - 1;
                    const float end = (xe >= 0 && xe < dx) ? me[(DIR > 0) ? 4 * q + 4 : 4 * q - 1] : kFarSentinel;
                    float res[4];
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        const int j = (DIR > 0) ? jj : 3 - jj;
                        const float down = (DIR > 0) ? ((j < 3) ? cur[j + 1] : end) : ((j > 0) ? cur[j - 1] : end);
                        float u;
                        if constexpr (NB) u = godunov_ref_nb(fminf(prev, down), ay[j], az[j], h, m2h, na3);
                        else u = godunov<RULE>(fminf(prev, down), ay[j], az[j], h);
                        const bool lo = u < cur[j];
                        res[j] = lo ? u : cur[j];
                        ch |= lo;
                        prev = res[j];
                    }
                    reinterpret_cast<float4*>(drow)[q] = make_float4(res[0], res[1], res[2], res[3]);
                }
            } else {
                // the lattice's last, partial chunk
#pragma unroll 1
                for (int jj = 0; jj < kXW; ++jj) {
                    const int j = (DIR > 0) ? jj : kXW - 1 - jj;
                    const int x = xc + j;
                    if (x >= dx) continue;
                    const float cur = me[j];
                    const float down = (x + DIR >= 0 && x + DIR < dx) ? me[j + DIR] : kFarSentinel;
                    const float ayj = min3f(yl[j], yh[j], kFarSentinel);
                    const float azj = min3f(zl[j], zh[j], kFarSentinel);
                    float u;
                    if constexpr (NB) u = godunov_ref_nb(fminf(prev, down), ayj, azj, h, m2h, na3);
                    else u = godunov<RULE>(fminf(prev, down), ayj, azj, h);
                    const bool lo = u < cur;
                    const float out = lo ? u : cur;
                    ch |= lo;
                    drow[j] = out;
                    prev = out;
                }
            }
        }
        __syncwarp();
        if (ty == 0) mbar_arrive(&empty[ci % kXWS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- y and z walks, TMA batches on a warp-specialised pipeline ------------------------
// The lines, tile (32 x 16 lines, two per thread) and per-line arithmetic of
// sweep_walk_kernel; the slices come in batches of 4, one cp.async.bulk.tensor copy per
// batch issued by a producer warp into a ring of kWPS slots with full / empty mbarriers.
// A batch box spans x0 - 4 .. x0 + 35 (its x start stays 16-byte aligned; the one-cell
// halo sits at columns 3 and 36), 18 rows and 4 slices; out-of-lattice cells arrive as
// NaN and the neighbour-pair minimum with the far sentinel turns them into it.
constexpr int kWPX = 40;                               // box columns
constexpr int kWPB = 4;                                // slices per batch
constexpr int kWPS = 4;                                // ring slots
constexpr int kWPBox = kWPX * kWHR * kWPB;             // floats per batch (2880)
constexpr int kWPSlotBytes = (kWPBox * 4 + 1023) / 1024 * 1024;  // batch bytes rounded up to 1 KB
constexpr int kWPThreads = kWThreads + 32;             // 8 consumer warps + 1 producer warp
constexpr size_t kWPSmem = (size_t)kWPS * kWPSlotBytes + 128 + 1024;

template <int AXIS, int RULE, int DIR>
__global__ void __launch_bounds__(kWPThreads) sweep_walk_pipe_kernel(const __grid_constant__ CUtensorMap tm,
                                                                      float* __restrict__ dst, Lattice L,
                                                                      int round, DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kWPS * kWPSlotBytes);
    uint64_t* empty = full + kWPS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const size_t plane = (size_t)L.px * dy;
    const int n_walk = (AXIS == 2) ? dz : dy;
    const int n_rows = (AXIS == 2) ? dy : dz;
    const size_t step_stride = (AXIS == 2) ? plane : (size_t)L.px;
    const size_t row_stride = (AXIS == 2) ? (size_t)L.px : plane;
    // shared-memory strides of a batch: box order is (x, y, z), x fastest
    constexpr int kSliceS = (AXIS == 2) ? kWHR * kWPX : kWPX;   // next slice
    constexpr int kRowS = (AXIS == 2) ? kWPX : kWPB * kWPX;     // next row
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * kWX, r0 = blockIdx.y * kWR;
    const int nbatches = (n_walk + kWPB - 1) / kWPB;
    if (tid == 0) {
        for (int s = 0; s < kWPS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kWThreads / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid >= kWThreads) {
        if (tid != kWThreads) return;
        int b = 0;
        for (; b < nbatches; ++b) {
            const int s = b % kWPS;
            if (b >= kWPS && !mbar_wait(&empty[s], ((b / kWPS) - 1) & 1, polls)) break;
            // lattice slices of this batch (walk order 4b .. 4b + 3)
            const int sl0 = (DIR > 0) ? b * kWPB : n_walk - kWPB - b * kWPB;
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kWPBox * 4);
            if (AXIS == 2) tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, r0 - 1, sl0, &full[s]);
            else tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, sl0, r0 - 1, &full[s]);
        }
        // let every copy still in flight land before the producer leaves (consumers that gave
        // up have left already); a break means the consumers stopped releasing slots
        for (int k = max(0, b - kWPS); k < b; ++k) mbar_wait(&full[k % kWPS], (k / kWPS) & 1);
        if (b < nbatches) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int tx = tid & 31, tr = tid >> 5;
    const int x = x0 + tx;
    const int ra = r0 + tr, rb = r0 + tr + 8;
    const bool act_a = (x < dx) && (ra < n_rows), act_b = (x < dx) && (rb < n_rows);
    const float h = L.h;
    // element of line a in slice q (box order) is tile[q * kSliceS + ma]
    const int ma = (tr + 1) * kRowS + (tx + 4), mb = ma + 8 * kRowS;
    auto slice_ptr = [&](int s) -> const float* {  // s in walk order
        const int b = s / kWPB, q = s - b * kWPB;
        const int qb = (DIR > 0) ? q : (kWPB - 1 - q);
        return reinterpret_cast<const float*>(tsm + (b % kWPS) * kWPSlotBytes) + qb * kSliceS;
    };
    float prev_a = kFarSentinel, prev_b = kFarSentinel;
    float cur_a = 0.0f, cur_b = 0.0f;
    bool ch = false;
    const long long sstep = (DIR > 0) ? (long long)step_stride : -(long long)step_stride;
    float* pa = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)ra * row_stride + x;
    float* pb = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)rb * row_stride + x;
#pragma unroll 1
    for (int b = 0; b < nbatches; ++b) {
        bool ok = mbar_wait(&full[b % kWPS], (b / kWPS) & 1, polls);
        if (ok && b + 1 < nbatches) ok = mbar_wait(&full[(b + 1) % kWPS], ((b + 1) / kWPS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if (tx == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        if (b == 0) {
            cur_a = slice_ptr(0)[ma];
            cur_b = slice_ptr(0)[mb];
        }
#pragma unroll
        for (int q = 0; q < kWPB; ++q) {
            const int s = b * kWPB + q;
            if (s >= n_walk) break;
            const float* cs = slice_ptr(s);
            const bool has_next = (s + 1 < n_walk);
            const float* ns = has_next ? slice_ptr(s + 1) : cs;
            const float nxt_a = has_next ? ns[ma] : kFarSentinel;
            const float nxt_b = has_next ? ns[mb] : kFarSentinel;
            if (act_a) {
                const float ax = fminf(fminf(cs[ma - 1], cs[ma + 1]), kFarSentinel);
                const float ar = fminf(fminf(cs[ma - kRowS], cs[ma + kRowS]), kFarSentinel);
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
                const float ax = fminf(fminf(cs[mb - 1], cs[mb + 1]), kFarSentinel);
                const float ar = fminf(fminf(cs[mb - kRowS], cs[mb + kRowS]), kFarSentinel);
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
        __syncwarp();
        if (tx == 0) mbar_arrive(&empty[b % kWPS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- y and z walks, TMA batches, four adjacent lines per thread ----------------------
// sweep_walk_pipe_kernel's tile (32 x 16 lines), boxes and barriers with 4 consumer warps
// and a 3-slot ring (more CTAs per SM): a thread walks the lines of 4 adjacent x in one
// row, so a slice costs it one 16-byte shared load of the next slice, two of the
// neighbouring rows, two scalar loads of the x neighbours at the quad's ends and one
// 16-byte global store -- 1.5 memory instructions per voxel where one line per thread
// issues 6 -- and the four branch-free updates interleave. Needs dim x a multiple of 4
// (as the TMA boxes do) and a 16-byte aligned destination, so quads are all in or all out.
constexpr int kWVConsumers = 128;
constexpr int kWVThreads = kWVConsumers + 32;
constexpr int kWVS = 3;                                // ring slots
constexpr size_t kWVSmem = (size_t)kWVS * kWPSlotBytes + 128 + 1024;

template <int AXIS, int RULE, int DIR>
__global__ void __launch_bounds__(kWVThreads) sweep_walk_vec_kernel(const __grid_constant__ CUtensorMap tm,
                                                                     float* __restrict__ dst, Lattice L,
                                                                     int round, DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kWVS * kWPSlotBytes);
    uint64_t* empty = full + kWVS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const size_t plane = (size_t)L.px * dy;
    const int n_walk = (AXIS == 2) ? dz : dy;
    const int n_rows = (AXIS == 2) ? dy : dz;
    const size_t step_stride = (AXIS == 2) ? plane : (size_t)L.px;
    const size_t row_stride = (AXIS == 2) ? (size_t)L.px : plane;
    constexpr int kSliceS = (AXIS == 2) ? kWHR * kWPX : kWPX;
    constexpr int kRowS = (AXIS == 2) ? kWPX : kWPB * kWPX;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * kWX, r0 = blockIdx.y * kWR;
    const int nbatches = (n_walk + kWPB - 1) / kWPB;
    if (tid == 0) {
        for (int s = 0; s < kWVS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kWVConsumers / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid >= kWVConsumers) {
        if (tid != kWVConsumers) return;
        int b = 0;
        for (; b < nbatches; ++b) {
            const int s = b % kWVS;
            if (b >= kWVS && !mbar_wait(&empty[s], ((b / kWVS) - 1) & 1, polls)) break;
            const int sl0 = (DIR > 0) ? b * kWPB : n_walk - kWPB - b * kWPB;
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kWPBox * 4);
            if (AXIS == 2) tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, r0 - 1, sl0, &full[s]);
            else tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, sl0, r0 - 1, &full[s]);
        }
        // let every copy still in flight land before the producer leaves (consumers that gave
        // up have left already); a break means the consumers stopped releasing slots
        for (int k = max(0, b - kWVS); k < b; ++k) mbar_wait(&full[k % kWVS], (k / kWVS) & 1);
        if (b < nbatches) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int cx = tid & 7, tr = tid >> 3;       // quad of x, row
    const int x = x0 + 4 * cx, r = r0 + tr;
    const bool act = (x < dx) && (r < n_rows);  // dim x is a multiple of 4: the quad is all in
    const float h = L.h;
    const int m = (tr + 1) * kRowS + 4 * cx + 4;  // 16-byte aligned: kRowS, kSliceS are multiples of 4
    auto slice_ptr = [&](int s) -> const float* {
        const int b = s / kWPB, q = s - b * kWPB;
        const int qb = (DIR > 0) ? q : (kWPB - 1 - q);
        return reinterpret_cast<const float*>(tsm + (b % kWVS) * kWPSlotBytes) + qb * kSliceS;
    };
    float prev[4] = {kFarSentinel, kFarSentinel, kFarSentinel, kFarSentinel};
    float cur[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    bool ch = false;
    const long long sstep = (DIR > 0) ? (long long)step_stride : -(long long)step_stride;
    float* p = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)r * row_stride + x;
#pragma unroll 1
    for (int b = 0; b < nbatches; ++b) {
        bool ok = mbar_wait(&full[b % kWVS], (b / kWVS) & 1, polls);
        if (ok && b + 1 < nbatches) ok = mbar_wait(&full[(b + 1) % kWVS], ((b + 1) / kWVS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if ((tid & 31) == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        if (b == 0) {
            const float4 c = *reinterpret_cast<const float4*>(slice_ptr(0) + m);
            cur[0] = c.x; cur[1] = c.y; cur[2] = c.z; cur[3] = c.w;
        }
#pragma unroll
        for (int q = 0; q < kWPB; ++q) {
            const int s = b * kWPB + q;
            if (s >= n_walk) break;
            const float* cs = slice_ptr(s);
            float nxt[4] = {kFarSentinel, kFarSentinel, kFarSentinel, kFarSentinel};
            if (s + 1 < n_walk) {
                const float4 n4 = *reinterpret_cast<const float4*>(slice_ptr(s + 1) + m);
                nxt[0] = n4.x; nxt[1] = n4.y; nxt[2] = n4.z; nxt[3] = n4.w;
            }
            if (act) {
                const float4 rm = *reinterpret_cast<const float4*>(cs + m - kRowS);
                const float4 rp = *reinterpret_cast<const float4*>(cs + m + kRowS);
                const float xl = cs[m - 1], xr = cs[m + 4];
                const float rmv[4] = {rm.x, rm.y, rm.z, rm.w}, rpv[4] = {rp.x, rp.y, rp.z, rp.w};
                float out[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float left = (j == 0) ? xl : cur[j - 1];
                    const float right = (j == 3) ? xr : cur[j + 1];
                    const float ax = fminf(fminf(left, right), kFarSentinel);
                    const float ar = fminf(fminf(rmv[j], rpv[j]), kFarSentinel);
                    const float al = fminf(prev[j], nxt[j]);
                    const float u = (AXIS == 2) ? godunov_sel<RULE>(ax, ar, al, h)
                                                : godunov_sel<RULE>(ax, al, ar, h);
                    out[j] = cur[j];
                    if (u < cur[j]) {
                        out[j] = u;
                        ch = true;
                    }
                    prev[j] = out[j];
                }
                *reinterpret_cast<float4*>(p) = make_float4(out[0], out[1], out[2], out[3]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) cur[j] = nxt[j];
            p += sstep;
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&empty[b % kWVS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// ---- y and z walks, four adjacent lines per thread, updates in packed pairs ----------
// sweep_walk_vec_kernel (tile, boxes, pipeline, loads and stores) for the reference's
// update with lines 0-1 and 2-3 of a thread's quad updated together by
// godunov_ref_pair on packed FP32 pairs (same roundings, half the arithmetic issue
// slots), and without the far-sentinel clamps of the neighbour minima, which a lattice
// with dim x a multiple of 4 and at least two rows across the walk never needs.
template <int AXIS, int DIR>
__global__ void __launch_bounds__(kWVThreads) sweep_walk_vec2_kernel(const __grid_constant__ CUtensorMap tm,
                                                                     float* __restrict__ dst, Lattice L,
                                                                     int round, DevState* ds) {
    if (ds->stop) return;
    const int polls = wait_poll_limit(ds);
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(tsm + kWVS * kWPSlotBytes);
    uint64_t* empty = full + kWVS;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const size_t plane = (size_t)L.px * dy;
    const int n_walk = (AXIS == 2) ? dz : dy;
    const int n_rows = (AXIS == 2) ? dy : dz;
    const size_t step_stride = (AXIS == 2) ? plane : (size_t)L.px;
    const size_t row_stride = (AXIS == 2) ? (size_t)L.px : plane;
    constexpr int kSliceS = (AXIS == 2) ? kWHR * kWPX : kWPX;
    constexpr int kRowS = (AXIS == 2) ? kWPX : kWPB * kWPX;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * kWX, r0 = blockIdx.y * kWR;
    const int nbatches = (n_walk + kWPB - 1) / kWPB;
    if (tid == 0) {
        for (int s = 0; s < kWVS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kWVConsumers / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid >= kWVConsumers) {
        if (tid != kWVConsumers) return;
        int b = 0;
        for (; b < nbatches; ++b) {
            const int s = b % kWVS;
            if (b >= kWVS && !mbar_wait(&empty[s], ((b / kWVS) - 1) & 1, polls)) break;
            const int sl0 = (DIR > 0) ? b * kWPB : n_walk - kWPB - b * kWPB;
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(&full[s], kWPBox * 4);
            if (AXIS == 2) tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, r0 - 1, sl0, &full[s]);
            else tma_load_3d(tsm + s * kWPSlotBytes, &tm, x0 - 4, sl0, r0 - 1, &full[s]);
        }
        // let every copy still in flight land before the producer leaves (consumers that gave
        // up have left already); a break means the consumers stopped releasing slots
        for (int k = max(0, b - kWVS); k < b; ++k) mbar_wait(&full[k % kWVS], (k / kWVS) & 1);
        if (b < nbatches) atomicAdd(&ds->wait_timeouts, 1ull);
        return;
    }
    const int cx = tid & 7, tr = tid >> 3;       // quad of x, row
    const int x = x0 + 4 * cx, r = r0 + tr;
    const bool act = (x < dx) && (r < n_rows);  // dim x is a multiple of 4: the quad is all in
    const GodunovPairConsts gc = godunov_pair_consts(L.h);
    const int m = (tr + 1) * kRowS + 4 * cx + 4;  // 16-byte aligned: kRowS, kSliceS are multiples of 4
    auto slice_ptr = [&](int s) -> const float* {
        const int b = s / kWPB, q = s - b * kWPB;
        const int qb = (DIR > 0) ? q : (kWPB - 1 - q);
        return reinterpret_cast<const float*>(tsm + (b % kWVS) * kWPSlotBytes) + qb * kSliceS;
    };
    float prev[4] = {kFarSentinel, kFarSentinel, kFarSentinel, kFarSentinel};
    float cur[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    bool ch = false;
    const long long sstep = (DIR > 0) ? (long long)step_stride : -(long long)step_stride;
    float* p = dst + (size_t)((DIR > 0) ? 0 : n_walk - 1) * step_stride + (size_t)r * row_stride + x;
#pragma unroll 1
    for (int b = 0; b < nbatches; ++b) {
        bool ok = mbar_wait(&full[b % kWVS], (b / kWVS) & 1, polls);
        if (ok && b + 1 < nbatches) ok = mbar_wait(&full[(b + 1) % kWVS], ((b + 1) / kWVS) & 1, polls);
        if (!__all_sync(0xffffffffu, ok)) {
            if ((tid & 31) == 0) atomicAdd(&ds->wait_timeouts, 1ull);
            return;
        }
        if (b == 0) {
            const float4 c = *reinterpret_cast<const float4*>(slice_ptr(0) + m);
            cur[0] = c.x; cur[1] = c.y; cur[2] = c.z; cur[3] = c.w;
        }
#pragma unroll
        for (int q = 0; q < kWPB; ++q) {
            const int s = b * kWPB + q;
            if (s >= n_walk) break;
            const float* cs = slice_ptr(s);
            float nxt[4] = {kFarSentinel, kFarSentinel, kFarSentinel, kFarSentinel};
            if (s + 1 < n_walk) {
                const float4 n4 = *reinterpret_cast<const float4*>(slice_ptr(s + 1) + m);
                nxt[0] = n4.x; nxt[1] = n4.y; nxt[2] = n4.z; nxt[3] = n4.w;
            }
            if (act) {
                const float4 rm = *reinterpret_cast<const float4*>(cs + m - kRowS);
                const float4 rp = *reinterpret_cast<const float4*>(cs + m + kRowS);
                const float xl = cs[m - 1], xr = cs[m + 4];
                const float rmv[4] = {rm.x, rm.y, rm.z, rm.w}, rpv[4] = {rp.x, rp.y, rp.z, rp.w};
                float ax[4], ar[4], al[4], u[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // no far-sentinel clamps: an out-of-lattice NaN always meets an
                    // in-lattice partner here (dim x a multiple of 4, at least 2 rows)
                    ax[j] = fminf((j == 0) ? xl : cur[j - 1], (j == 3) ? xr : cur[j + 1]);
                    ar[j] = fminf(rmv[j], rpv[j]);
                    al[j] = fminf(prev[j], nxt[j]);
                }
#pragma unroll
                for (int j = 0; j < 4; j += 2) {
                    if (AXIS == 2) godunov_ref_pair(ax[j], ar[j], al[j], ax[j + 1], ar[j + 1], al[j + 1], gc, u[j], u[j + 1]);
                    else godunov_ref_pair(ax[j], al[j], ar[j], ax[j + 1], al[j + 1], ar[j + 1], gc, u[j], u[j + 1]);
                }
                float out[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    out[j] = cur[j];
                    if (u[j] < cur[j]) {
                        out[j] = u[j];
                        ch = true;
                    }
                    prev[j] = out[j];
                }
                *reinterpret_cast<float4*>(p) = make_float4(out[0], out[1], out[2], out[3]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) cur[j] = nxt[j];
            p += sstep;
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&empty[b % kWVS]);
    }
    mark_changed(ch, &ds->changed[round]);
}

// Layout check of the staged tile: one CTA loads the box at (x, y, z) of a grid whose
// cells hold their own linear index, and every thread compares elements (scalar reads
// through tsw, vector reads through tvec) with the expected value or NaN outside.
__global__ void selftest_tma_kernel(const __grid_constant__ CUtensorMap tm, int x, int y, int z, int dx, int dy,
                                    int dz, unsigned long long* mism) {
    extern __shared__ unsigned char tsm_raw[];
    unsigned char* tsm = align1k(tsm_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + kTSlotBytes);
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_expect_tx(bar, kTBox * 4);
        tma_load_3d(tsm, &tm, x, y, z, bar);
        s_ok = mbar_wait(bar, 0) ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) {
        if (threadIdx.x == 0) atomicAdd(mism, 1000000ull);
        return;
    }
    const float* tile = reinterpret_cast<const float*>(tsm);
    unsigned long long bad = 0;
    for (int e = threadIdx.x; e < kTBox; e += blockDim.x) {
        const int r = e / kXC, j = e % kXC;
        const int gx = x + j, gy = y + r % kXHY, gz = z + r / kXHY;
        const bool inb = gx >= 0 && gx < dx && gy >= 0 && gy < dy && gz >= 0 && gz < dz;
        const float want = inb ? (float)(((long long)gz * dy + gy) * dx + gx) : 0.0f;
        const float got = tile[tsw(r, j)];
        const float4 v = tvec(tile, r, j >> 2);
        const float gv = (j & 3) == 0 ? v.x : (j & 3) == 1 ? v.y : (j & 3) == 2 ? v.z : v.w;
        if (inb ? (got != want || gv != want) : (got == got || gv == gv)) ++bad;
    }
    if (bad) atomicAdd(mism, bad);
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
// surf_tol (world units, negative = off): voxels this close to the surface take the exact-
// arithmetic sign of a point on it (inside) -- the exact-signs modes.
__global__ void __launch_bounds__(256) apply_kernel(const float* __restrict__ g, const uint32_t* __restrict__ sbits,
                                                    Lattice L, float* __restrict__ out, const DevState* ds,
                                                    float surf_tol) {
    if (ds->verify_state != 1 || ds->abort_ || ds->wait_timeouts) return;
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
                    cudaStream_t st, const GridMap* src_map, int xsched, int wsched) {
    const bool tma = src_map && src_map->valid;
    if (xsched == 0) xsched = tma ? kXTmaPipe : kXCpAsync;
    if (!tma) xsched = kXCpAsync;
    const bool wtma = src_map && src_map->walk_valid;
    if (wsched == 0) wsched = wtma ? kWTmaPipe : kWCpAsync;
    if (!wtma) wsched = kWCpAsync;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    GBSDF_COUNT_LAUNCH();
    // four lines per thread: 16-byte stores need an aligned destination (rows already are)
    if ((wsched == kWTmaVec || wsched == kWTmaVec2) && (reinterpret_cast<uintptr_t>(dst) & 15)) wsched = kWTmaPipe;
    // packed pairs: the reference's update, at least two rows across the walk, and a voxel
    // size whose square-root operands stay where nsqrt2_rn is exact
    const bool pair_ok = (RULE == 0) && pair_sqrt_ok(L.h);
    if (wsched == kWTmaVec2 && (!pair_ok || (axis == 2 ? dy : dz) < 2)) wsched = kWTmaVec;
    if (axis != 0 && wsched == kWTmaVec2) {
        const int n_rows = (axis == 2) ? dy : dz;
        dim3 grid((dx + kWX - 1) / kWX, (n_rows + kWR - 1) / kWR);
        if (axis == 2) {
            cudaFuncSetAttribute(sweep_walk_vec2_kernel<2, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWVSmem);
            sweep_walk_vec2_kernel<2, DIR><<<grid, kWVThreads, kWVSmem, st>>>(src_map->zmap, dst, L, round, ds);
        } else {
            cudaFuncSetAttribute(sweep_walk_vec2_kernel<1, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWVSmem);
            sweep_walk_vec2_kernel<1, DIR><<<grid, kWVThreads, kWVSmem, st>>>(src_map->ymap, dst, L, round, ds);
        }
    } else if (axis != 0 && wsched == kWTmaVec) {
        const int n_rows = (axis == 2) ? dy : dz;
        dim3 grid((dx + kWX - 1) / kWX, (n_rows + kWR - 1) / kWR);
        if (axis == 2) {
            cudaFuncSetAttribute(sweep_walk_vec_kernel<2, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWVSmem);
            sweep_walk_vec_kernel<2, RULE, DIR><<<grid, kWVThreads, kWVSmem, st>>>(src_map->zmap, dst, L, round,
                                                                                 ds);
        } else {
            cudaFuncSetAttribute(sweep_walk_vec_kernel<1, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWVSmem);
            sweep_walk_vec_kernel<1, RULE, DIR><<<grid, kWVThreads, kWVSmem, st>>>(src_map->ymap, dst, L, round,
                                                                                 ds);
        }
    } else if (axis != 0 && wsched == kWTmaPipe) {
        const int n_rows = (axis == 2) ? dy : dz;
        dim3 grid((dx + kWX - 1) / kWX, (n_rows + kWR - 1) / kWR);
        if (axis == 2) {
            cudaFuncSetAttribute(sweep_walk_pipe_kernel<2, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWPSmem);
            sweep_walk_pipe_kernel<2, RULE, DIR><<<grid, kWPThreads, kWPSmem, st>>>(src_map->zmap, dst, L, round,
                                                                                  ds);
        } else {
            cudaFuncSetAttribute(sweep_walk_pipe_kernel<1, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWPSmem);
            sweep_walk_pipe_kernel<1, RULE, DIR><<<grid, kWPThreads, kWPSmem, st>>>(src_map->ymap, dst, L, round,
                                                                                  ds);
        }
    } else if (axis == 2) {
        dim3 grid((dx + kWX - 1) / kWX, (dy + kWR - 1) / kWR);
        cudaFuncSetAttribute(sweep_walk_kernel<2, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kWSmem);
        sweep_walk_kernel<2, RULE, DIR><<<grid, kWThreads, kWSmem, st>>>(src, dst, L, round, ds);
    } else if (axis == 1) {
        dim3 grid((dx + kWX - 1) / kWX, (dz + kWR - 1) / kWR);
        cudaFuncSetAttribute(sweep_walk_kernel<1, RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kWSmem);
        sweep_walk_kernel<1, RULE, DIR><<<grid, kWThreads, kWSmem, st>>>(src, dst, L, round, ds);
    } else if (xsched == kXTmaPipe2 && pair_ok && dy >= 2 && dz >= 2) {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        cudaFuncSetAttribute(sweep_x_pipe2_kernel<DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPSmem);
        sweep_x_pipe2_kernel<DIR><<<grid, kP2Threads, kPSmem, st>>>(src_map->map, dst, L, round, ds);
    } else if (xsched == kXTmaWide && src_map->wide_valid) {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        if (pair_ok) {
            cudaFuncSetAttribute(sweep_x_wide_kernel<0, DIR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kXWSmem);
            sweep_x_wide_kernel<0, DIR, true><<<grid, kPThreads, kXWSmem, st>>>(src_map->wmap, dst, L, round, ds);
        } else {
            cudaFuncSetAttribute(sweep_x_wide_kernel<RULE, DIR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kXWSmem);
            sweep_x_wide_kernel<RULE, DIR, false><<<grid, kPThreads, kXWSmem, st>>>(src_map->wmap, dst, L, round,
                                                                                   ds);
        }
    } else if (xsched == kXTmaPipe || xsched == kXTmaPipe2 || xsched == kXTmaWide) {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        if (pair_ok) {
            cudaFuncSetAttribute(sweep_x_pipe_kernel<0, DIR, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kPSmem);
            sweep_x_pipe_kernel<0, DIR, 2><<<grid, kPThreads, kPSmem, st>>>(src_map->map, dst, L, round, ds);
        } else {
            cudaFuncSetAttribute(sweep_x_pipe_kernel<RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kPSmem);
            sweep_x_pipe_kernel<RULE, DIR><<<grid, kPThreads, kPSmem, st>>>(src_map->map, dst, L, round, ds);
        }
    } else if (xsched == kXTmaRing) {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        cudaFuncSetAttribute(sweep_x_tma_kernel<RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kTSmem);
        sweep_x_tma_kernel<RULE, DIR><<<grid, kXThreads, kTSmem, st>>>(src_map->map, dst, L, round, ds);
    } else {
        dim3 grid((dy + kXY - 1) / kXY, (dz + kXZ - 1) / kXZ);
        cudaFuncSetAttribute(sweep_x_kernel<RULE, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kXSmem);
        sweep_x_kernel<RULE, DIR><<<grid, kXThreads, kXSmem, st>>>(src, dst, L, round, ds);
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tiled_encoder() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return static_cast<EncodeTiledFn>(nullptr);
        }
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// A 3D tiled descriptor of a grid of dx x dy x dz voxels whose rows are px floats apart.
bool encode_box(CUtensorMap* m, const float* base, int dx, int dy, int dz, int px, int bx = kXC, int by = kXHY,
                int bz = kXHZ, CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_32B) {
    EncodeTiledFn fn = tiled_encoder();
    if (!fn) return false;
    const cuuint64_t gdim[3] = {(cuuint64_t)dx, (cuuint64_t)dy, (cuuint64_t)dz};
    const cuuint64_t gstride[2] = {(cuuint64_t)px * 4, (cuuint64_t)px * dy * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), gdim, gstride, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA) == CUDA_SUCCESS;
}

}  // namespace

bool encode_grid_map(GridMap& m, const float* base, const Lattice& L) {
    m.valid = false;
    m.walk_valid = false;
    m.wide_valid = false;
    // row and plane pitches must be multiples of 16 bytes, the base 16-byte aligned
    if ((L.px & 3) != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    m.valid = encode_box(&m.map, base, dx, dy, dz, L.px);
    m.walk_valid = m.valid &&
                   encode_box(&m.ymap, base, dx, dy, dz, L.px, kWPX, kWPB, kWHR, CU_TENSOR_MAP_SWIZZLE_NONE) &&
                   encode_box(&m.zmap, base, dx, dy, dz, L.px, kWPX, kWHR, kWPB, CU_TENSOR_MAP_SWIZZLE_NONE);
    m.wide_valid = m.valid && encode_box(&m.wmap, base, dx, dy, dz, L.px, kXWB, kXHY, kXHZ,
                                         CU_TENSOR_MAP_SWIZZLE_NONE);
    return m.valid;
}

void launch_sweep(int rule, int axis, int dir, int round, const float* src, float* dst, const Lattice& L,
                  DevState* ds, cudaStream_t st, const GridMap* src_map, int x_schedule, int w_schedule) {
    if (rule == 0) {
        if (dir > 0) launch_sweep_t<0, 1>(axis, round, src, dst, L, ds, st, src_map, x_schedule, w_schedule);
        else launch_sweep_t<0, -1>(axis, round, src, dst, L, ds, st, src_map, x_schedule, w_schedule);
    } else {
        if (dir > 0) launch_sweep_t<1, 1>(axis, round, src, dst, L, ds, st, src_map, x_schedule, w_schedule);
        else launch_sweep_t<1, -1>(axis, round, src, dst, L, ds, st, src_map, x_schedule, w_schedule);
    }
}

int selftest_tma_tile(unsigned long long* mism_dev) {
    const int dx = 48, dy = 40, dz = 16;
    const size_t n = (size_t)dx * dy * dz;
    std::vector<float> hv(n);
    for (size_t i = 0; i < n; ++i) hv[i] = (float)i;
    float* g = nullptr;
    if (cudaMalloc(&g, n * 4) != cudaSuccess) return 1;
    int rc = 0;
    CUtensorMap m;
    if (cudaMemcpy(g, hv.data(), n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        !encode_box(&m, g, dx, dy, dz, dx)) {
        rc = 1;
    } else {
        const int pts[5][3] = {{0, -1, -1}, {8, 5, 3}, {40, 31, 7}, {16, 10, 0}, {32, -1, 12}};
        const size_t smem = kTSlotBytes + 64 + 1024;
        cudaFuncSetAttribute(selftest_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        for (auto& p : pts) selftest_tma_kernel<<<1, 256, smem>>>(m, p[0], p[1], p[2], dx, dy, dz, mism_dev);
        if (cudaDeviceSynchronize() != cudaSuccess) rc = 1;
    }
    cudaGetLastError();
    cudaFree(g);
    return rc;
}

namespace {
// Dense x-fastest grid (rows of dims[0]) <-> the sweeps' padded copy (rows of px floats;
// pad columns written as 0, never read as voxels). One warp per row at a time, no index
// division; 16-byte copies where dims[0] is a multiple of 4 (both rows' starts are then
// 16-byte aligned and a quad is wholly voxels or wholly pad).
template <bool VEC>
__global__ void pad_rows_kernel(const float* __restrict__ dense, float* __restrict__ pad, Lattice L) {
    const long long nrows = (long long)L.dims[1] * L.dims[2];
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31, dx = L.dims[0], px = L.px;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += nw) {
        const float* s = dense + r * dx;
        float* d = pad + r * px;
        if constexpr (VEC) {
            for (int q = lane; q < (px >> 2); q += 32)
                reinterpret_cast<float4*>(d)[q] =
                    (4 * q < dx) ? reinterpret_cast<const float4*>(s)[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            for (int x = lane; x < px; x += 32) d[x] = (x < dx) ? s[x] : 0.0f;
        }
    }
}
// The copy back, counting on the way the voxels still at the far sentinel (the audit,
// [D2]) when `far` is not null.
template <bool VEC>
__global__ void unpad_rows_kernel(const float* __restrict__ pad, float* __restrict__ dense, Lattice L,
                                  unsigned long long* __restrict__ far) {
    const long long nrows = (long long)L.dims[1] * L.dims[2];
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31, dx = L.dims[0], px = L.px;
    unsigned c = 0;
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += nw) {
        const float* s = pad + r * px;
        float* d = dense + r * dx;
        if constexpr (VEC) {
            for (int q = lane; q < (dx >> 2); q += 32) {
                const float4 v = reinterpret_cast<const float4*>(s)[q];
                reinterpret_cast<float4*>(d)[q] = v;
                c += (v.x >= 1e29f) + (v.y >= 1e29f) + (v.z >= 1e29f) + (v.w >= 1e29f);
            }
        } else {
            for (int x = lane; x < dx; x += 32) {
                const float v = s[x];
                d[x] = v;
                c += (v >= 1e29f);
            }
        }
    }
    if (far) {
        c = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0 && c) atomicAdd(far, (unsigned long long)c);
    }
}

unsigned row_copy_blocks(const Lattice& P) {
    const long long nrows = (long long)P.dims[1] * P.dims[2];
    return (unsigned)std::max<long long>(1, std::min<long long>((nrows + 7) / 8, 152LL * 16));
}
}  // namespace

void launch_pad_rows(const float* dense, float* pad, const Lattice& P, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    if ((P.dims[0] & 3) == 0) pad_rows_kernel<true><<<row_copy_blocks(P), 256, 0, st>>>(dense, pad, P);
    else pad_rows_kernel<false><<<row_copy_blocks(P), 256, 0, st>>>(dense, pad, P);
}
void launch_unpad_rows(const float* pad, float* dense, const Lattice& P, cudaStream_t st, DevState* audit_ds) {
    GBSDF_COUNT_LAUNCH();
    unsigned long long* far = audit_ds ? &audit_ds->far_residual : nullptr;
    if ((P.dims[0] & 3) == 0) unpad_rows_kernel<true><<<row_copy_blocks(P), 256, 0, st>>>(pad, dense, P, far);
    else unpad_rows_kernel<false><<<row_copy_blocks(P), 256, 0, st>>>(pad, dense, P, far);
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
