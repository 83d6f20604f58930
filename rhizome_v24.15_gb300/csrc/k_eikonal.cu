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

constexpr int kZX = 32, kZY = 8;  // z/y sweeps: CTA = 32 (x) x 8 lines

__device__ __forceinline__ void mark_changed(bool ch, int* flag) {
    unsigned b = __ballot_sync(__activemask(), ch);
    if (b && (threadIdx.x & 31) == __ffs(b) - 1) *flag = 1;
}

template <int RULE>
__global__ void __launch_bounds__(kZX* kZY) sweep_z_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                            Lattice L, int dir, int round, DevState* ds) {
    if (ds->stop) return;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const int x = blockIdx.x * kZX + threadIdx.x, y = blockIdx.y * kZY + threadIdx.y;
    if (x >= dx || y >= dy) return;
    const float h = L.h;
    const size_t plane = (size_t)dx * dy;
    const size_t col = (size_t)y * dx + x;
    int z = (dir > 0) ? 0 : dz - 1;
    float cur = src[(size_t)z * plane + col];
    float prev = kFarSentinel;
    bool ch = false;
    for (int s = 0; s < dz; ++s) {
        const size_t idx = (size_t)z * plane + col;
        const int zn = z + dir;
        const float nxt = (zn >= 0 && zn < dz) ? src[idx + (dir > 0 ? plane : (size_t)0 - plane)] : kFarSentinel;
        const float xm = (x > 0) ? src[idx - 1] : kFarSentinel;
        const float xp = (x < dx - 1) ? src[idx + 1] : kFarSentinel;
        const float ym = (y > 0) ? src[idx - dx] : kFarSentinel;
        const float yp = (y < dy - 1) ? src[idx + dx] : kFarSentinel;
        const float az = fminf(prev, nxt);
        const float u = godunov<RULE>(fminf(xm, xp), fminf(ym, yp), az, h);
        float out = cur;
        if (u < cur) {
            out = u;
            ch = true;
        }
        dst[idx] = out;
        prev = out;
        cur = nxt;
        z = zn;
    }
    mark_changed(ch, &ds->changed[round]);
}

template <int RULE>
__global__ void __launch_bounds__(kZX* kZY) sweep_y_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                            Lattice L, int dir, int round, DevState* ds) {
    if (ds->stop) return;
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const int x = blockIdx.x * kZX + threadIdx.x, z = blockIdx.y * kZY + threadIdx.y;
    if (x >= dx || z >= dz) return;
    const float h = L.h;
    const size_t plane = (size_t)dx * dy;
    const size_t line = (size_t)z * plane + x;
    int y = (dir > 0) ? 0 : dy - 1;
    float cur = src[line + (size_t)y * dx];
    float prev = kFarSentinel;
    bool ch = false;
    for (int s = 0; s < dy; ++s) {
        const size_t idx = line + (size_t)y * dx;
        const int yn = y + dir;
        const float nxt = (yn >= 0 && yn < dy) ? src[idx + (dir > 0 ? (size_t)dx : (size_t)0 - (size_t)dx)]
                                               : kFarSentinel;
        const float xm = (x > 0) ? src[idx - 1] : kFarSentinel;
        const float xp = (x < dx - 1) ? src[idx + 1] : kFarSentinel;
        const float zm = (z > 0) ? src[idx - plane] : kFarSentinel;
        const float zp = (z < dz - 1) ? src[idx + plane] : kFarSentinel;
        const float ay = fminf(prev, nxt);
        const float u = godunov<RULE>(fminf(xm, xp), ay, fminf(zm, zp), h);
        float out = cur;
        if (u < cur) {
            out = u;
            ch = true;
        }
        dst[idx] = out;
        prev = out;
        cur = nxt;
        y = yn;
    }
    mark_changed(ch, &ds->changed[round]);
}

constexpr int kXLY = 16, kXLZ = 8;            // lines per CTA of the x sweep
constexpr int kXC = 32;                        // voxels per chunk
constexpr int kXS = 35;                        // padded line stride in shared memory
constexpr int kXLines = (kXLY + 2) * (kXLZ + 2);  // staged lines incl. halo (180)
constexpr int kXThreads = kXLY * kXLZ;         // 128

template <int RULE>
__global__ void __launch_bounds__(kXThreads) sweep_x_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                             Lattice L, int dir, int round, DevState* ds) {
    if (ds->stop) return;
    __shared__ float tile[kXLines * kXS];
    __shared__ float outt[kXThreads * (kXC + 1)];
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    const float h = L.h;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int y0 = blockIdx.x * kXLY, z0 = blockIdx.y * kXLZ;
    const int ly = tid % kXLY, lz = tid / kXLY;
    const int y = y0 + ly, z = z0 + lz;
    const bool valid = (y < dy) && (z < dz);
    const int nchunks = (dx + kXC - 1) / kXC;
    const size_t plane = (size_t)dx * dy;
    float prev = kFarSentinel;
    bool ch = false;
    // own line and its 4 cross neighbours in the staged tile
    const int me = (lz + 1) * (kXLY + 2) + (ly + 1);
    const int n_ym = me - 1, n_yp = me + 1, n_zm = me - (kXLY + 2), n_zp = me + (kXLY + 2);
    for (int ci = 0; ci < nchunks; ++ci) {
        const int c = (dir > 0) ? ci : (nchunks - 1 - ci);
        const int xc = c * kXC;
        // ---- stage x in [xc-1, xc+32] of the 180 lines (coalesced 128-byte rows)
        for (int ln = warp; ln < kXLines; ln += kXThreads / 32) {
            const int ty = ln % (kXLY + 2), tz = ln / (kXLY + 2);
            const int yy = y0 - 1 + ty, zz = z0 - 1 + tz;
            const bool lok = (yy >= 0 && yy < dy && zz >= 0 && zz < dz);
            const size_t base = (size_t)zz * plane + (size_t)yy * dx;
            const int xa = xc + lane;
            tile[ln * kXS + 1 + lane] = (lok && xa < dx) ? src[base + xa] : kFarSentinel;
            if (lane < 2) {
                const int xe = (lane == 0) ? xc - 1 : xc + kXC;
                const int slot = (lane == 0) ? 0 : kXC + 1;
                tile[ln * kXS + slot] = (lok && xe >= 0 && xe < dx) ? src[base + xe] : kFarSentinel;
            }
        }
        __syncthreads();
        if (valid) {
            for (int j = 0; j < kXC; ++j) {
                const int xi = (dir > 0) ? j : (kXC - 1 - j);
                const int x = xc + xi;
                if (x >= dx) continue;
                const int i = xi + 1;
                const float cur = tile[me * kXS + i];
                const float down = tile[me * kXS + i + dir];
                const float ax = fminf(prev, down);
                const float ay = fminf(tile[n_ym * kXS + i], tile[n_yp * kXS + i]);
                const float az = fminf(tile[n_zm * kXS + i], tile[n_zp * kXS + i]);
                const float u = godunov<RULE>(ax, ay, az, h);
                float out = cur;
                if (u < cur) {
                    out = u;
                    ch = true;
                }
                outt[tid * (kXC + 1) + xi] = out;
                prev = out;
            }
        }
        __syncthreads();
        // ---- store the chunk (coalesced rows)
        for (int ln = warp; ln < kXThreads; ln += kXThreads / 32) {
            const int yy = y0 + ln % kXLY, zz = z0 + ln / kXLY;
            const int xa = xc + lane;
            if (yy < dy && zz < dz && xa < dx) dst[(size_t)zz * plane + (size_t)yy * dx + xa] = outt[ln * (kXC + 1) + lane];
        }
        __syncthreads();
    }
    if (valid) {
        if (ch) ds->changed[round] = 1;
    }
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

__device__ __forceinline__ bool sign_bit(const uint32_t* sbits, const Lattice& L, long long i) {
    long long dx = L.dims[0];
    long long row = i / dx;
    int x = (int)(i - row * dx);
    return (sbits[(size_t)row * L.wx + (x >> 5)] >> (x & 31)) & 1u;
}

// [D3] cuda_rasterizer.cu:544-556: leftover sentinels -> -band / +band by the signs of
// that moment (runs only when the audit found a residual).
__global__ void clamp_kernel(float* __restrict__ g, const uint32_t* __restrict__ sbits, Lattice L, DevState* ds) {
    if (ds->far_residual == 0) return;
    const float bw = (float)kBandVoxels * L.h;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.N; i += stride)
        if (g[i] >= 1e29f) g[i] = sign_bit(sbits, L, i) ? -bw : bw;
}

// [F] cuda_rasterizer.cu:650-661, applied only when the verify loop came back clean
// (on divergence the output stays untouched, cuda_rasterizer.cu:788-791).
__global__ void apply_kernel(const float* __restrict__ g, const uint32_t* __restrict__ sbits, Lattice L,
                             float* __restrict__ out, const DevState* ds) {
    if (ds->verify_state != 1) return;
    const long long dx = L.dims[0];
    long long stride = (long long)gridDim.x * blockDim.x;
    // one thread per 4 consecutive voxels of a row where possible
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.N; i += stride) {
        float d = g[i];
        if (d > 1e29f) d = 1e6f;
        long long row = i / dx;
        int x = (int)(i - row * dx);
        bool in = (sbits[(size_t)row * L.wx + (x >> 5)] >> (x & 31)) & 1u;
        out[i] = in ? -d : d;
    }
}

}  // namespace

void launch_sweep(int rule, int axis, int dir, int round, const float* src, float* dst, const Lattice& L,
                  DevState* ds, cudaStream_t st) {
    const int dx = L.dims[0], dy = L.dims[1], dz = L.dims[2];
    if (axis == 2) {
        dim3 grid((dx + kZX - 1) / kZX, (dy + kZY - 1) / kZY), block(kZX, kZY);
        if (rule == 0) { GBSDF_COUNT_LAUNCH(); sweep_z_kernel<0><<<grid, block, 0, st>>>(src, dst, L, dir, round, ds); }
        else { GBSDF_COUNT_LAUNCH(); sweep_z_kernel<1><<<grid, block, 0, st>>>(src, dst, L, dir, round, ds); }
    } else if (axis == 1) {
        dim3 grid((dx + kZX - 1) / kZX, (dz + kZY - 1) / kZY), block(kZX, kZY);
        if (rule == 0) { GBSDF_COUNT_LAUNCH(); sweep_y_kernel<0><<<grid, block, 0, st>>>(src, dst, L, dir, round, ds); }
        else { GBSDF_COUNT_LAUNCH(); sweep_y_kernel<1><<<grid, block, 0, st>>>(src, dst, L, dir, round, ds); }
    } else {
        dim3 grid((dy + kXLY - 1) / kXLY, (dz + kXLZ - 1) / kXLZ);
        if (rule == 0) { GBSDF_COUNT_LAUNCH(); sweep_x_kernel<0><<<grid, kXThreads, 0, st>>>(src, dst, L, dir, round, ds); }
        else { GBSDF_COUNT_LAUNCH(); sweep_x_kernel<1><<<grid, kXThreads, 0, st>>>(src, dst, L, dir, round, ds); }
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
    long long blocks = std::min<long long>((L.N + 255) / 256, 152LL * 16);
    GBSDF_COUNT_LAUNCH();
    clamp_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, sbits, L, ds);
}

void launch_apply(const float* g, const uint32_t* sbits, const Lattice& L, float* out, const DevState* ds,
                  cudaStream_t st) {
    long long blocks = std::min<long long>((L.N + 255) / 256, 152LL * 32);
    GBSDF_COUNT_LAUNCH();
    apply_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, sbits, L, out, ds);
}

}  // namespace gbsdf
