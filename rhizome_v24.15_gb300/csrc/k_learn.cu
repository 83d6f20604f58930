// k_learn.cu — learned sign-risk proposals: per-brick features, a 32 -> 64 -> 64 -> 1
// MLP with BF16 weights and FP32 accumulation (forward, backward, Adam), and the
// proposal step that hands the riskiest 8^3 bricks to the exact winding kernel.
//
// No counterpart in the reference (its fast path verifies signs only by stratified
// probes, cuda_rasterizer.cu:566-646). The network never supplies a sign: it only
// chooses which bricks the exact winding kernel re-decides.
//
// Parameter layout (FP32 master copy, 6337 floats):
//   W1 [64][32] | b1 [64] | W2 [64][64] | b2 [64] | w3 [64] | b3 [1]
// Matrix products round weights and activations to BF16 (round to nearest even) and
// accumulate in FP32; biases stay FP32.
#include <cuda_bf16.h>

#include <algorithm>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

namespace {

constexpr int kF = kMlpIn, kH = kMlpHidden;
constexpr int oW1 = 0, ob1 = oW1 + kH * kF, oW2 = ob1 + kH, ob2 = oW2 + kH * kH, ow3 = ob2 + kH, ob3 = ow3 + kH;
static_assert(ob3 + 1 == kMlpParams, "parameter layout");

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---- open (boundary) edges: hash of the two endpoints' positions -------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long edge_key(const float* a, const float* b) {
    // order the endpoints lexicographically so both triangles of an edge agree
    bool swap = (a[0] > b[0]) || (a[0] == b[0] && (a[1] > b[1] || (a[1] == b[1] && a[2] > b[2])));
    const float* p = swap ? b : a;
    const float* q = swap ? a : b;
    unsigned long long k = 0x243f6a8885a308d3ull;
    for (int i = 0; i < 3; ++i) k = mix64(k ^ __float_as_uint(p[i]));
    for (int i = 0; i < 3; ++i) k = mix64(k ^ ((unsigned long long)__float_as_uint(q[i]) << 1));
    return k ? k : 1ull;
}

__global__ void edge_insert_kernel(const float* __restrict__ t12, long long T, unsigned long long* __restrict__ keys,
                                   unsigned* __restrict__ counts, unsigned long long cap) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * T) return;
    const long long t = e / 3;
    const int k = (int)(e - 3 * t);
    const float* v = t12 + 12 * t;
    const unsigned long long key = edge_key(v + 3 * k, v + 3 * ((k + 1) % 3));
    unsigned long long slot = key & (cap - 1);
    for (unsigned long long probe = 0; probe < cap; ++probe) {
        const unsigned long long prev = atomicCAS(&keys[slot], 0ull, key);
        if (prev == 0ull || prev == key) {
            atomicAdd(&counts[slot], 1u);
            return;
        }
        slot = (slot + 1) & (cap - 1);
    }
}

__global__ void edge_open_kernel(const float* __restrict__ t12, long long T, const unsigned long long* __restrict__ keys,
                                 const unsigned* __restrict__ counts, unsigned long long cap, Lattice L,
                                 unsigned* __restrict__ open_count) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * T) return;
    const long long t = e / 3;
    const int k = (int)(e - 3 * t);
    const float* v = t12 + 12 * t;
    const float* a = v + 3 * k;
    const float* b = v + 3 * ((k + 1) % 3);
    const unsigned long long key = edge_key(a, b);
    unsigned long long slot = key & (cap - 1);
    for (unsigned long long probe = 0; probe < cap; ++probe) {
        const unsigned long long kk = keys[slot];
        if (kk == key) {
            if (counts[slot] != 1u) return;  // shared by two (or more) triangles
            int bidx[3];
            for (int i = 0; i < 3; ++i) {
                const float m = 0.5f * (a[i] + b[i]);
                const int c = (int)floorf(m / L.h + 0.5f) - L.mn[i];
                if (c < 0 || c >= L.dims[i]) return;
                bidx[i] = c / kBrick;
            }
            atomicAdd(&open_count[((long long)bidx[2] * L.nb[1] + bidx[1]) * L.nb[0] + bidx[0]], 1u);
            return;
        }
        if (kk == 0ull) return;
        slot = (slot + 1) & (cap - 1);
    }
}

// ---- per-brick base features ---------------------------------------------------------
// One CTA of 64 threads per brick; thread t reads the 8-voxel x-row (y = t % 8, z = t / 8).
// Computed after the plain path's verify / patch stage, from the unsigned distance field,
// the current signs S, the mask E of voxels already decided by the exact winding number,
// and a signed-crossing parity pass (S2, with U2 its unknown columns):
// base[0..7] = log1p(triangles binned to the brick), log1p(open edges),
//              log1p(voxels decided exactly), log1p(voxels not decided exactly where the
//              sign and the signed crossings disagree), log1p(voxels within the +-8h band),
//              log1p(inside voxels), min(|d| / h, 8) / 8, log1p(voxels with |d| < h / 2)
__global__ void __launch_bounds__(64) brick_base_kernel(const float* __restrict__ dist, const uint32_t* __restrict__ S,
                                                        const uint32_t* __restrict__ E, const uint32_t* __restrict__ S2,
                                                        const uint32_t* __restrict__ U2,
                                                        const unsigned* __restrict__ brick_tris,
                                                        const unsigned* __restrict__ open_count, Lattice L,
                                                        float* __restrict__ base) {
    const long long b = blockIdx.x;
    const int nbx = L.nb[0], nby = L.nb[1];
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    const int t = threadIdx.x;
    const int y = by * kBrick + (t & 7), z = bz * kBrick + (t >> 3);
    const int x0 = bx * kBrick;
    const float h = L.h;
    const float band = (float)kBandVoxels * h;
    int c_unk = 0, c_diff = 0, c_band = 0, c_in = 0, c_near = 0;
    float dmin = 8.0f * h;
    if (y < L.dims[1] && z < L.dims[2]) {
        const size_t row = (size_t)z * L.dims[1] + y;
        const float* dr = dist + row * L.dims[0];
        const size_t w = row * L.wx + (x0 >> 5);
        const int sh = x0 & 31;
        const uint32_t sb = S[w] >> sh, ub = E[w] >> sh, s2 = S2[w] >> sh, u2 = U2[w] >> sh;
        for (int j = 0; j < kBrick; ++j) {
            const int x = x0 + j;
            if (x >= L.dims[0]) break;
            const float d = dr[x];
            const bool inb = d <= band;
            c_band += inb;
            c_near += (d < 0.5f * h);
            dmin = fminf(dmin, d);
            const bool uu = (ub >> j) & 1u, uu2 = (u2 >> j) & 1u;
            c_unk += uu;
            c_in += (sb >> j) & 1u;
            c_diff += (!uu && !uu2 && (((sb ^ s2) >> j) & 1u));
        }
    }
    // block reduction (2 warps)
    __shared__ int red[5][2];
    __shared__ float redf[2];
    const int lane = t & 31, wp = t >> 5;
    int v[5] = {c_unk, c_diff, c_band, c_in, c_near};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        v[i] = __reduce_add_sync(0xffffffffu, v[i]);
        if (lane == 0) red[i][wp] = v[i];
    }
    float m = dmin;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) redf[wp] = m;
    __syncthreads();
    if (t == 0) {
        float* o = base + b * kBrickBase;
        o[0] = log1pf((float)brick_tris[b]);
        o[1] = log1pf((float)open_count[b]);
        o[2] = log1pf((float)(red[0][0] + red[0][1]));
        o[3] = log1pf((float)(red[1][0] + red[1][1]));
        o[4] = log1pf((float)(red[2][0] + red[2][1]));
        o[5] = log1pf((float)(red[3][0] + red[3][1]));
        o[6] = fminf(fminf(redf[0], redf[1]) / h, 8.0f) / 8.0f;
        o[7] = log1pf((float)(red[4][0] + red[4][1]));
    }
}

// ---- 32 features per brick: base, 6-neighbour sum, 26-neighbour max, 5^3 mean ---------
__global__ void brick_features_kernel(const float* __restrict__ base, Lattice L, float* __restrict__ X) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= L.nbricks) return;
    const int nbx = L.nb[0], nby = L.nb[1], nbz = L.nb[2];
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    float f6[kBrickBase], f26[kBrickBase], f125[kBrickBase];
    for (int i = 0; i < kBrickBase; ++i) f6[i] = f26[i] = f125[i] = 0.0f;
    int n125 = 0;
    for (int dz = -2; dz <= 2; ++dz)
        for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
                const int x = bx + dx, y = by + dy, z = bz + dz;
                if (x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
                const float* q = base + (((long long)z * nby + y) * nbx + x) * kBrickBase;
                const int ad = abs(dx) + abs(dy) + abs(dz);
                const int mx = max(abs(dx), max(abs(dy), abs(dz)));
                ++n125;
                for (int i = 0; i < kBrickBase; ++i) {
                    const float vv = q[i];
                    f125[i] += vv;
                    if (ad == 1) f6[i] += vv;
                    if (mx == 1) f26[i] = fmaxf(f26[i], vv);
                }
            }
    float* o = X + b * kMlpIn;
    const float* q = base + b * kBrickBase;
    for (int i = 0; i < kBrickBase; ++i) {
        o[i] = q[i];
        o[kBrickBase + i] = f6[i] / 6.0f;
        o[2 * kBrickBase + i] = f26[i];
        o[3 * kBrickBase + i] = f125[i] / (float)max(n125, 1);
    }
}

// ---- MLP forward on the tensor cores ------------------------------------------------
// Warp-level mma.sync m16n8k16 (BF16 x BF16 -> FP32), one warp per 16 samples at a time.
// Layer 1 (16 x 32 by 32 x 64) is 8 column tiles x 2 k-steps. Its FP32 accumulators, with
// bias, ReLU and BF16 rounding, are layer 2's A operand as they stand: the accumulator
// layout of two adjacent 8-column tiles (rows g and g+8, columns 2t and 2t+1 of each) is
// the operand layout of one 16-deep k-step, so activations never leave registers. Layer
// 2 (16 x 64 by 64 x 64) is 8 x 4 mma; the 64-wide output product is summed per thread and
// across the 4 threads of a row. Products of BF16 values are exact in FP32; the sums run in
// the tensor cores' FP32 accumulation order, not the sequential order of a scalar loop.
// Weights are staged once per CTA as BF16 rows at padded strides (40 and 72 elements), at
// which the 32 lanes' operand loads fall in 32 distinct banks.
constexpr int kMmaThreads = 128;
constexpr int kW1S = 40, kW2S = 72;

// Two FP32 values rounded to BF16 (to nearest even) in one register, lo in the low half.
__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(kMmaThreads) mlp_forward_kernel(const float* __restrict__ P,
                                                                 const float* __restrict__ X, long long B,
                                                                 float* __restrict__ logits) {
    __shared__ __align__(16) __nv_bfloat16 sW1[kH * kW1S];
    __shared__ __align__(16) __nv_bfloat16 sW2[kH * kW2S];
    __shared__ float sb1[kH], sb2[kH], sw3[kH];
    __shared__ float sb3;
    for (int i = threadIdx.x; i < kH * kF; i += blockDim.x)
        sW1[(i / kF) * kW1S + (i % kF)] = __float2bfloat16_rn(P[oW1 + i]);
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x)
        sW2[(i / kH) * kW2S + (i % kH)] = __float2bfloat16_rn(P[oW2 + i]);
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        sb1[i] = P[ob1 + i];
        sb2[i] = P[ob2 + i];
        sw3[i] = bf(P[ow3 + i]);
    }
    if (threadIdx.x == 0) sb3 = P[ob3];
    __syncthreads();
    const uint32_t* w1 = reinterpret_cast<const uint32_t*>(sW1);
    const uint32_t* w2 = reinterpret_cast<const uint32_t*>(sW2);
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long ntiles = (B + 15) / 16;
    const long long wstride = (long long)gridDim.x * (kMmaThreads / 32);
    for (long long tile = (long long)blockIdx.x * (kMmaThreads / 32) + (threadIdx.x >> 5); tile < ntiles;
         tile += wstride) {
        const long long r0 = tile * 16 + g, r1 = r0 + 8;
        const bool v0 = r0 < B, v1 = r1 < B;
        // layer 1 operand: the features rounded to BF16 (rows past the end read as 0)
        uint32_t a[2][4];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int c = 16 * s + 2 * t;
            const float2 z2 = make_float2(0.0f, 0.0f);
            const float2 x00 = v0 ? *reinterpret_cast<const float2*>(X + r0 * kF + c) : z2;
            const float2 x10 = v1 ? *reinterpret_cast<const float2*>(X + r1 * kF + c) : z2;
            const float2 x01 = v0 ? *reinterpret_cast<const float2*>(X + r0 * kF + c + 8) : z2;
            const float2 x11 = v1 ? *reinterpret_cast<const float2*>(X + r1 * kF + c + 8) : z2;
            a[s][0] = pack_bf2(x00.x, x00.y);
            a[s][1] = pack_bf2(x10.x, x10.y);
            a[s][2] = pack_bf2(x01.x, x01.y);
            a[s][3] = pack_bf2(x11.x, x11.y);
        }
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const int n = 8 * j + g;
#pragma unroll
            for (int s = 0; s < 2; ++s)
                mma_bf16(acc[j], a[s], w1[(n * kW1S + 16 * s + 2 * t) >> 1], w1[(n * kW1S + 16 * s + 8 + 2 * t) >> 1]);
        }
        // bias, ReLU, BF16: the four k-steps of layer 2's operand
        uint32_t hf[4][4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int j = 2 * s + q, col = 8 * j + 2 * t;
                hf[s][2 * q] = pack_bf2(fmaxf(acc[j][0] + sb1[col], 0.0f), fmaxf(acc[j][1] + sb1[col + 1], 0.0f));
                hf[s][2 * q + 1] =
                    pack_bf2(fmaxf(acc[j][2] + sb1[col], 0.0f), fmaxf(acc[j][3] + sb1[col + 1], 0.0f));
            }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const int n = 8 * j + g;
#pragma unroll
            for (int s = 0; s < 4; ++s)
                mma_bf16(acc[j], hf[s], w2[(n * kW2S + 16 * s + 2 * t) >> 1], w2[(n * kW2S + 16 * s + 8 + 2 * t) >> 1]);
        }
        // output layer: this thread's 16 columns of rows g and g+8, then the row's 4 threads
        float z0 = 0.0f, z1 = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int col = 8 * j + 2 * t;
            z0 = __fmaf_rn(sw3[col], bf(fmaxf(acc[j][0] + sb2[col], 0.0f)), z0);
            z0 = __fmaf_rn(sw3[col + 1], bf(fmaxf(acc[j][1] + sb2[col + 1], 0.0f)), z0);
            z1 = __fmaf_rn(sw3[col], bf(fmaxf(acc[j][2] + sb2[col], 0.0f)), z1);
            z1 = __fmaf_rn(sw3[col + 1], bf(fmaxf(acc[j][3] + sb2[col + 1], 0.0f)), z1);
        }
        z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
        z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
        z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
        z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
        if (t == 0) {
            if (v0) logits[r0] = z0 + sb3;
            if (v1) logits[r1] = z1 + sb3;
        }
    }
}

// ---- MLP backward on the tensor cores: weighted binary cross-entropy with logits -----
// One CTA of 4 warps takes kMlpBwdSamples = 64 samples, 16 per warp, and writes one
// partial gradient; mlp_reduce_kernel sums the partials in CTA order, so gradients are
// deterministic. Phase 1, each warp for its 16 samples: the forward pass as in
// mlp_forward_kernel (mma), the loss and dL/dz, dZ2 = dL/dz * w3 where z2 > 0, and
// dA1 = dZ2 W2 on the tensor cores straight from the accumulator layout (as the forward
// pass chains its layers), dZ1 = dA1 where z1 > 0; the column sums for db1, db2, dw3, db3
// by butterflies over the rows. The factors of the weight gradients go to shared memory
// transposed, sample index fastest: A1, X (BF16, exactly the forward pass's rounded
// values), dZ2 and dZ1 as BF16 high and low parts (hi = RN_bf16(v), lo = RN_bf16(v - hi),
// so a product with a BF16 operand keeps about 16 bits). Phase 2, warp w: its 16 rows of
// dW2 = dZ2^T A1 and dW1 = dZ1^T X over the 64 samples (mma, hi and lo terms).
constexpr int kBwdThreads = 128;
constexpr int kTS = 72;  // padded row stride (BF16) of the transposed factors, 64 samples + 8
constexpr int kBwdSmemBytes =
    (kH * kW1S + 2 * kH * kW2S + kH * kTS + kF * kTS + 4 * kH * kTS) * 2 + (3 * kH + 4 * (3 * kH + 2) + 4) * 4;
static_assert(kMlpBwdSamples == 64, "one 64-sample step per CTA");

__device__ __forceinline__ uint32_t ld_bf2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// hi / lo BF16 split of v
__device__ __forceinline__ void split_bf(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(v);
    lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// Sum over the 8 row groups (lanes with equal lane % 4): every lane ends with its column's total.
__device__ __forceinline__ float rows_sum(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

__global__ void __launch_bounds__(kBwdThreads) mlp_backward_kernel(const float* __restrict__ P,
                                                                   const float* __restrict__ X,
                                                                   const float* __restrict__ y,
                                                                   const float* __restrict__ wt, long long B,
                                                                   float* __restrict__ partial,
                                                                   float* __restrict__ loss_partial) {
    extern __shared__ __align__(16) unsigned char bsm[];
    __nv_bfloat16* sW1 = reinterpret_cast<__nv_bfloat16*>(bsm);   // [64][kW1S]  W1[j][c]
    __nv_bfloat16* sW2 = sW1 + kH * kW1S;                          // [64][kW2S]  W2[j][i]
    __nv_bfloat16* sW2T = sW2 + kH * kW2S;                         // [64][kW2S]  W2[j][i] at [i][j]
    __nv_bfloat16* sA1T = sW2T + kH * kW2S;                        // [64 i][kTS] samples
    __nv_bfloat16* sXT = sA1T + kH * kTS;                          // [32 c][kTS]
    __nv_bfloat16* sD2h = sXT + kF * kTS;                          // [64 j][kTS]
    __nv_bfloat16* sD2l = sD2h + kH * kTS;
    __nv_bfloat16* sD1h = sD2l + kH * kTS;
    __nv_bfloat16* sD1l = sD1h + kH * kTS;
    float* sb1 = reinterpret_cast<float*>(sD1l + kH * kTS);
    float* sb2 = sb1 + kH;
    float* sw3 = sb2 + kH;
    float* vred = sw3 + kH;  // [4 warps][db1 64 | db2 64 | dw3 64 | db3 | loss]
    constexpr int kV = 3 * kH + 2;
    for (int i = threadIdx.x; i < kH * kF; i += blockDim.x)
        sW1[(i / kF) * kW1S + (i % kF)] = __float2bfloat16_rn(P[oW1 + i]);
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) {
        const __nv_bfloat16 v = __float2bfloat16_rn(P[oW2 + i]);
        sW2[(i / kH) * kW2S + (i % kH)] = v;
        sW2T[(i % kH) * kW2S + (i / kH)] = v;
    }
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        sb1[i] = P[ob1 + i];
        sb2[i] = P[ob2 + i];
        sw3[i] = bf(P[ow3 + i]);
    }
    __syncthreads();
    const float b3 = P[ob3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int q0 = 16 * warp + g, q1 = q0 + 8;  // this thread's two samples within the CTA's 64
    const long long r0 = (long long)blockIdx.x * kMlpBwdSamples + q0, r1 = r0 + 8;
    const bool v0 = r0 < B, v1 = r1 < B;
    // ---- phase 1: forward, loss, back-propagation through the layers -----------------
    uint32_t a[2][4];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int c = 16 * s + 2 * t;
        const float2 z2v = make_float2(0.0f, 0.0f);
        const float2 x00 = v0 ? *reinterpret_cast<const float2*>(X + r0 * kF + c) : z2v;
        const float2 x10 = v1 ? *reinterpret_cast<const float2*>(X + r1 * kF + c) : z2v;
        const float2 x01 = v0 ? *reinterpret_cast<const float2*>(X + r0 * kF + c + 8) : z2v;
        const float2 x11 = v1 ? *reinterpret_cast<const float2*>(X + r1 * kF + c + 8) : z2v;
        a[s][0] = pack_bf2(x00.x, x00.y);
        a[s][1] = pack_bf2(x10.x, x10.y);
        a[s][2] = pack_bf2(x01.x, x01.y);
        a[s][3] = pack_bf2(x11.x, x11.y);
        const __nv_bfloat16* e0 = reinterpret_cast<const __nv_bfloat16*>(&a[s][0]);
        const __nv_bfloat16* e1 = reinterpret_cast<const __nv_bfloat16*>(&a[s][1]);
        const __nv_bfloat16* e2 = reinterpret_cast<const __nv_bfloat16*>(&a[s][2]);
        const __nv_bfloat16* e3 = reinterpret_cast<const __nv_bfloat16*>(&a[s][3]);
        sXT[c * kTS + q0] = e0[0];
        sXT[(c + 1) * kTS + q0] = e0[1];
        sXT[c * kTS + q1] = e1[0];
        sXT[(c + 1) * kTS + q1] = e1[1];
        sXT[(c + 8) * kTS + q0] = e2[0];
        sXT[(c + 9) * kTS + q0] = e2[1];
        sXT[(c + 8) * kTS + q1] = e3[0];
        sXT[(c + 9) * kTS + q1] = e3[1];
    }
    const uint32_t* w1 = reinterpret_cast<const uint32_t*>(sW1);
    const uint32_t* w2 = reinterpret_cast<const uint32_t*>(sW2);
    const uint32_t* w2t = reinterpret_cast<const uint32_t*>(sW2T);
    float z1[8][4];  // layer-1 pre-activations
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        z1[j][0] = z1[j][1] = z1[j][2] = z1[j][3] = 0.0f;
        const int n = 8 * j + g;
#pragma unroll
        for (int s = 0; s < 2; ++s)
            mma_bf16(z1[j], a[s], w1[(n * kW1S + 16 * s + 2 * t) >> 1], w1[(n * kW1S + 16 * s + 8 + 2 * t) >> 1]);
        const int col = 8 * j + 2 * t;
        z1[j][0] += sb1[col];
        z1[j][1] += sb1[col + 1];
        z1[j][2] += sb1[col];
        z1[j][3] += sb1[col + 1];
    }
    uint32_t hf[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int j = 2 * s + q, col = 8 * j + 2 * t;
            hf[s][2 * q] = pack_bf2(fmaxf(z1[j][0], 0.0f), fmaxf(z1[j][1], 0.0f));
            hf[s][2 * q + 1] = pack_bf2(fmaxf(z1[j][2], 0.0f), fmaxf(z1[j][3], 0.0f));
            const __nv_bfloat16* u = reinterpret_cast<const __nv_bfloat16*>(&hf[s][2 * q]);
            const __nv_bfloat16* l = reinterpret_cast<const __nv_bfloat16*>(&hf[s][2 * q + 1]);
            sA1T[col * kTS + q0] = u[0];
            sA1T[(col + 1) * kTS + q0] = u[1];
            sA1T[col * kTS + q1] = l[0];
            sA1T[(col + 1) * kTS + q1] = l[1];
        }
    float z2[8][4];  // layer-2 pre-activations
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        z2[j][0] = z2[j][1] = z2[j][2] = z2[j][3] = 0.0f;
        const int n = 8 * j + g;
#pragma unroll
        for (int s = 0; s < 4; ++s)
            mma_bf16(z2[j], hf[s], w2[(n * kW2S + 16 * s + 2 * t) >> 1], w2[(n * kW2S + 16 * s + 8 + 2 * t) >> 1]);
        const int col = 8 * j + 2 * t;
        z2[j][0] += sb2[col];
        z2[j][1] += sb2[col + 1];
        z2[j][2] += sb2[col];
        z2[j][3] += sb2[col + 1];
    }
    float zo0 = 0.0f, zo1 = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int col = 8 * j + 2 * t;
        zo0 = __fmaf_rn(sw3[col], bf(fmaxf(z2[j][0], 0.0f)), zo0);
        zo0 = __fmaf_rn(sw3[col + 1], bf(fmaxf(z2[j][1], 0.0f)), zo0);
        zo1 = __fmaf_rn(sw3[col], bf(fmaxf(z2[j][2], 0.0f)), zo1);
        zo1 = __fmaf_rn(sw3[col + 1], bf(fmaxf(z2[j][3], 0.0f)), zo1);
    }
    zo0 += __shfl_xor_sync(0xffffffffu, zo0, 1);
    zo1 += __shfl_xor_sync(0xffffffffu, zo1, 1);
    zo0 += __shfl_xor_sync(0xffffffffu, zo0, 2);
    zo1 += __shfl_xor_sync(0xffffffffu, zo1, 2);
    zo0 += b3;
    zo1 += b3;
    // loss and dL/dz (rows past the end contribute nothing)
    float dz0 = 0.0f, dz1 = 0.0f, lsum = 0.0f;
    if (v0) {
        const float yy = y[r0], ww = wt ? wt[r0] : 1.0f;
        lsum += ww * (fmaxf(zo0, 0.0f) - zo0 * yy + log1pf(expf(-fabsf(zo0))));
        dz0 = ww * (1.0f / (1.0f + expf(-zo0)) - yy);
    }
    if (v1) {
        const float yy = y[r1], ww = wt ? wt[r1] : 1.0f;
        lsum += ww * (fmaxf(zo1, 0.0f) - zo1 * yy + log1pf(expf(-fabsf(zo1))));
        dz1 = ww * (1.0f / (1.0f + expf(-zo1)) - yy);
    }
    // dZ2, its column sums (db2) and dw3 = sum dz * a2; dZ2 as layer-back A operand and
    // transposed hi / lo factors
    float* vr = vred + warp * kV;
    uint32_t dh[4][4], dl[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int col = 8 * j + 2 * t;
        float d[4];
        d[0] = z2[j][0] > 0.0f ? dz0 * sw3[col] : 0.0f;
        d[1] = z2[j][1] > 0.0f ? dz0 * sw3[col + 1] : 0.0f;
        d[2] = z2[j][2] > 0.0f ? dz1 * sw3[col] : 0.0f;
        d[3] = z2[j][3] > 0.0f ? dz1 * sw3[col + 1] : 0.0f;
        const float c0 = rows_sum(d[0] + d[2]), c1 = rows_sum(d[1] + d[3]);
        const float w0 = rows_sum(dz0 * bf(fmaxf(z2[j][0], 0.0f)) + dz1 * bf(fmaxf(z2[j][2], 0.0f)));
        const float w1v = rows_sum(dz0 * bf(fmaxf(z2[j][1], 0.0f)) + dz1 * bf(fmaxf(z2[j][3], 0.0f)));
        if (g == 0) {
            vr[kH + col] = c0;
            vr[kH + col + 1] = c1;
            vr[2 * kH + col] = w0;
            vr[2 * kH + col + 1] = w1v;
        }
        __nv_bfloat16 hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split_bf(d[e], hi[e], lo[e]);
        sD2h[col * kTS + q0] = hi[0];
        sD2h[(col + 1) * kTS + q0] = hi[1];
        sD2h[col * kTS + q1] = hi[2];
        sD2h[(col + 1) * kTS + q1] = hi[3];
        sD2l[col * kTS + q0] = lo[0];
        sD2l[(col + 1) * kTS + q0] = lo[1];
        sD2l[col * kTS + q1] = lo[2];
        sD2l[(col + 1) * kTS + q1] = lo[3];
        const int s = j >> 1, q = j & 1;
        dh[s][2 * q] = pack_bf2(__bfloat162float(hi[0]), __bfloat162float(hi[1]));
        dh[s][2 * q + 1] = pack_bf2(__bfloat162float(hi[2]), __bfloat162float(hi[3]));
        dl[s][2 * q] = pack_bf2(__bfloat162float(lo[0]), __bfloat162float(lo[1]));
        dl[s][2 * q + 1] = pack_bf2(__bfloat162float(lo[2]), __bfloat162float(lo[3]));
    }
    {
        const float d3 = rows_sum(dz0 + dz1);
        const float ls = rows_sum(t == 0 ? lsum : 0.0f);
        if (lane == 0) {
            vr[3 * kH] = d3;
            vr[3 * kH + 1] = ls;
        }
    }
    // dA1 = dZ2 W2 (B operand: W2 transposed, rows i), dZ1 = dA1 where z1 > 0
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const int n = 8 * m + g;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t b0 = w2t[(n * kW2S + 16 * s + 2 * t) >> 1], b1 = w2t[(n * kW2S + 16 * s + 8 + 2 * t) >> 1];
            mma_bf16(acc, dh[s], b0, b1);
            mma_bf16(acc, dl[s], b0, b1);
        }
        const int col = 8 * m + 2 * t;
        float d[4];
        d[0] = z1[m][0] > 0.0f ? acc[0] : 0.0f;
        d[1] = z1[m][1] > 0.0f ? acc[1] : 0.0f;
        d[2] = z1[m][2] > 0.0f ? acc[2] : 0.0f;
        d[3] = z1[m][3] > 0.0f ? acc[3] : 0.0f;
        const float c0 = rows_sum(d[0] + d[2]), c1 = rows_sum(d[1] + d[3]);
        if (g == 0) {
            vr[col] = c0;
            vr[col + 1] = c1;
        }
        __nv_bfloat16 hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split_bf(d[e], hi[e], lo[e]);
        sD1h[col * kTS + q0] = hi[0];
        sD1h[(col + 1) * kTS + q0] = hi[1];
        sD1h[col * kTS + q1] = hi[2];
        sD1h[(col + 1) * kTS + q1] = hi[3];
        sD1l[col * kTS + q0] = lo[0];
        sD1l[(col + 1) * kTS + q0] = lo[1];
        sD1l[col * kTS + q1] = lo[2];
        sD1l[(col + 1) * kTS + q1] = lo[3];
    }
    __syncthreads();
    // ---- phase 2: this warp's 16 rows of dW2 and dW1 over the 64 samples -------------
    float* out = partial + (long long)blockIdx.x * kMlpParams;
    const int jr = 16 * warp + g;  // rows jr and jr + 8 of the slice
    uint32_t ah[4][4], al[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int k = 16 * s + 2 * t;
        ah[s][0] = ld_bf2(sD2h + jr * kTS + k);
        ah[s][1] = ld_bf2(sD2h + (jr + 8) * kTS + k);
        ah[s][2] = ld_bf2(sD2h + jr * kTS + k + 8);
        ah[s][3] = ld_bf2(sD2h + (jr + 8) * kTS + k + 8);
        al[s][0] = ld_bf2(sD2l + jr * kTS + k);
        al[s][1] = ld_bf2(sD2l + (jr + 8) * kTS + k);
        al[s][2] = ld_bf2(sD2l + jr * kTS + k + 8);
        al[s][3] = ld_bf2(sD2l + (jr + 8) * kTS + k + 8);
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const int n = 8 * m + g;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t b0 = ld_bf2(sA1T + n * kTS + 16 * s + 2 * t), b1 = ld_bf2(sA1T + n * kTS + 16 * s + 8 + 2 * t);
            mma_bf16(acc, ah[s], b0, b1);
            mma_bf16(acc, al[s], b0, b1);
        }
        const int col = 8 * m + 2 * t;
        out[oW2 + jr * kH + col] = acc[0];
        out[oW2 + jr * kH + col + 1] = acc[1];
        out[oW2 + (jr + 8) * kH + col] = acc[2];
        out[oW2 + (jr + 8) * kH + col + 1] = acc[3];
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int k = 16 * s + 2 * t;
        ah[s][0] = ld_bf2(sD1h + jr * kTS + k);
        ah[s][1] = ld_bf2(sD1h + (jr + 8) * kTS + k);
        ah[s][2] = ld_bf2(sD1h + jr * kTS + k + 8);
        ah[s][3] = ld_bf2(sD1h + (jr + 8) * kTS + k + 8);
        al[s][0] = ld_bf2(sD1l + jr * kTS + k);
        al[s][1] = ld_bf2(sD1l + (jr + 8) * kTS + k);
        al[s][2] = ld_bf2(sD1l + jr * kTS + k + 8);
        al[s][3] = ld_bf2(sD1l + (jr + 8) * kTS + k + 8);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const int n = 8 * m + g;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t b0 = ld_bf2(sXT + n * kTS + 16 * s + 2 * t), b1 = ld_bf2(sXT + n * kTS + 16 * s + 8 + 2 * t);
            mma_bf16(acc, ah[s], b0, b1);
            mma_bf16(acc, al[s], b0, b1);
        }
        const int col = 8 * m + 2 * t;
        out[oW1 + jr * kF + col] = acc[0];
        out[oW1 + jr * kF + col + 1] = acc[1];
        out[oW1 + (jr + 8) * kF + col] = acc[2];
        out[oW1 + (jr + 8) * kF + col + 1] = acc[3];
    }
    // the vector parts, summed over the 4 warps in order
    for (int i = threadIdx.x; i < kV; i += blockDim.x) {
        const float v = ((vred[i] + vred[kV + i]) + vred[2 * kV + i]) + vred[3 * kV + i];
        if (i < kH) out[ob1 + i] = v;
        else if (i < 2 * kH) out[ob2 + i - kH] = v;
        else if (i < 3 * kH) out[ow3 + i - 2 * kH] = v;
        else if (i == 3 * kH) out[ob3] = v;
        else loss_partial[blockIdx.x] = v;
    }
}

__global__ void mlp_reduce_kernel(const float* __restrict__ partial, const float* __restrict__ loss_partial,
                                  int nparts, float* __restrict__ grad, float* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpParams) {
        float s = 0.0f;
        for (int p = 0; p < nparts; ++p) s += partial[(long long)p * kMlpParams + i];
        grad[i] = s;
    }
    if (i == 0) {
        float s = 0.0f;
        for (int p = 0; p < nparts; ++p) s += loss_partial[p];
        *loss = s;
    }
}

__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float scale,
                            float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * scale;
    m[i] = b1 * m[i] + (1.0f - b1) * gi;
    v[i] = b2 * v[i] + (1.0f - b2) * gi * gi;
    P[i] -= lr * (m[i] / bc1) / (sqrtf(v[i] / bc2) + eps);
}

// ---- proposals: mark every voxel of a risky brick unknown (exact winding next) ---------
// Deterministic budget: bricks above the threshold are binned by logit (kPropBins bins of
// 1/kPropScale); the lowest bin whose bricks, together with all higher bins, still fit the
// budget is picked on the device, and every brick at or above it is proposed.
__device__ __forceinline__ int prop_bin(float logit, float thr) {
    return (int)fminf((float)(kPropBins - 1), (logit - thr) * kPropScale);
}

__global__ void propose_hist_kernel(const float* __restrict__ logits, long long nb, float logit_thr,
                                    unsigned* __restrict__ hist) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const float z = logits[b];
    if (!(z > logit_thr)) return;
    atomicAdd(&hist[prop_bin(z, logit_thr)], 1u);
}

// The budget's cut on the device, so a build needs no host round trip between scoring and
// proposing.
__global__ void propose_cut_kernel(const unsigned* __restrict__ hist, unsigned budget, int* __restrict__ cut) {
    unsigned long long total = 0;
    int c = 0;
    for (int b = kPropBins - 1; b >= 0; --b) {
        if (total + hist[b] > budget) {
            c = b + 1;
            break;
        }
        total += hist[b];
    }
    *cut = c;
}

__global__ void propose_dev_kernel(const float* __restrict__ logits, Lattice L, float logit_thr,
                                   const int* __restrict__ cut, unsigned* __restrict__ n_prop,
                                   uint32_t* __restrict__ U, const DevState* __restrict__ ds) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // after an escalation the signs are no longer the plain path's: nothing to aim at
    if (b >= L.nbricks || ds->escalated) return;
    const float z = logits[b];
    const int cut_bin = *cut;
    if (cut_bin >= kPropBins || !(z > logit_thr) || prop_bin(z, logit_thr) < cut_bin) return;
    atomicAdd(n_prop, 1u);
    const int nbx = L.nb[0], nby = L.nb[1];
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    const int x0 = bx * kBrick;
    const int nx = min(kBrick, L.dims[0] - x0);
    const uint32_t mask = ((nx >= 32) ? 0xffffffffu : ((1u << nx) - 1u)) << (x0 & 31);
    for (int z3 = bz * kBrick; z3 < min(L.dims[2], bz * kBrick + kBrick); ++z3)
        for (int y = by * kBrick; y < min(L.dims[1], by * kBrick + kBrick); ++y)
            atomicOr(&U[((size_t)z3 * L.dims[1] + y) * L.wx + (x0 >> 5)], mask);
}

// Escalation of a diverged verify (learned mode): the signs become the signed-crossing
// pass's (the winding number along near-lattice rays) and its unknown columns -- rays
// through holes -- are listed for the exact winding number. The decision is read by
// every block before the state is marked, in a kernel of its own.
__global__ void escalate_copy_kernel(const DevState* __restrict__ ds, uint32_t* __restrict__ S,
                                     uint32_t* __restrict__ U, const uint32_t* __restrict__ S2,
                                     const uint32_t* __restrict__ U2, long long nwords) {
    if (ds->verify_state == 1) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += stride) {
        S[i] = S2[i];
        U[i] = U2[i];
    }
}

__global__ void escalate_mark_kernel(DevState* ds) {
    if (ds->verify_state == 1) return;
    ds->escalated = 1;
    ds->verify_state = 1;
}

}  // namespace

void launch_propose_dev(const float* logits, const Lattice& L, float logit_thr, unsigned budget, unsigned* hist,
                        DevState* ds, uint32_t* U, cudaStream_t st) {
    if (L.nbricks <= 0) return;
    cudaMemsetAsync(hist, 0, (size_t)kPropBins * 4, st);
    launch_propose_hist(logits, L.nbricks, logit_thr, hist, st);
    GBSDF_COUNT_LAUNCH();
    propose_cut_kernel<<<1, 1, 0, st>>>(hist, budget, &ds->prop_cut);
    GBSDF_COUNT_LAUNCH();
    propose_dev_kernel<<<(unsigned)((L.nbricks + 255) / 256), 256, 0, st>>>(logits, L, logit_thr, &ds->prop_cut,
                                                                             &ds->proposed, U, ds);
}

void launch_escalate(DevState* ds, uint32_t* S, uint32_t* U, const uint32_t* S2, const uint32_t* U2,
                     const Lattice& L, int num_sms, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    const long long blocks = std::min<long long>((L.nwords + 255) / 256, (long long)num_sms * 8);
    escalate_copy_kernel<<<(unsigned)std::max<long long>(blocks, 1), 256, 0, st>>>(ds, S, U, S2, U2, L.nwords);
    GBSDF_COUNT_LAUNCH();
    escalate_mark_kernel<<<1, 1, 0, st>>>(ds);
}

long long edge_table_cap(long long T) {
    long long need = 6 * T + 1024, cap = 1024;
    while (cap < need) cap <<= 1;
    return cap;
}

void launch_open_edges(const float* t12, long long T, const Lattice& L, unsigned long long* keys, unsigned* counts,
                       long long cap, unsigned* open_count, cudaStream_t st) {
    if (T <= 0) return;
    const unsigned blocks = (unsigned)((3 * T + 255) / 256);
    GBSDF_COUNT_LAUNCH();
    edge_insert_kernel<<<blocks, 256, 0, st>>>(t12, T, keys, counts, (unsigned long long)cap);
    GBSDF_COUNT_LAUNCH();
    edge_open_kernel<<<blocks, 256, 0, st>>>(t12, T, keys, counts, (unsigned long long)cap, L, open_count);
}

void launch_brick_features(const float* dist, const uint32_t* S, const uint32_t* E, const uint32_t* S2,
                           const uint32_t* U2, const unsigned* brick_tris, const unsigned* open_count,
                           const Lattice& L, float* base, float* X, cudaStream_t st) {
    GBSDF_COUNT_LAUNCH();
    brick_base_kernel<<<(unsigned)L.nbricks, 64, 0, st>>>(dist, S, E, S2, U2, brick_tris, open_count, L, base);
    GBSDF_COUNT_LAUNCH();
    brick_features_kernel<<<(unsigned)((L.nbricks + 127) / 128), 128, 0, st>>>(base, L, X);
}

void launch_mlp_forward(const float* P, const float* X, long long B, float* logits, cudaStream_t st) {
    if (B <= 0) return;
    const long long tiles = (B + 15) / 16;
    const long long blocks = std::min<long long>((tiles + kMmaThreads / 32 - 1) / (kMmaThreads / 32), 152LL * 8);
    GBSDF_COUNT_LAUNCH();
    mlp_forward_kernel<<<(unsigned)blocks, kMmaThreads, 0, st>>>(P, X, B, logits);
}

int mlp_backward_parts(long long B) { return (int)((B + kMlpBwdSamples - 1) / kMlpBwdSamples); }

void launch_mlp_backward(const float* P, const float* X, const float* y, const float* wt, long long B, float* partial,
                         float* loss_partial, float* grad, float* loss, cudaStream_t st) {
    const int parts = mlp_backward_parts(B);
    if (parts <= 0) return;
    GBSDF_COUNT_LAUNCH();
    cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmemBytes);
    mlp_backward_kernel<<<parts, kBwdThreads, kBwdSmemBytes, st>>>(P, X, y, wt, B, partial, loss_partial);
    GBSDF_COUNT_LAUNCH();
    mlp_reduce_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(partial, loss_partial, parts, grad, loss);
}

void launch_adam(float* P, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                 float scale, int step, cudaStream_t st) {
    const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    GBSDF_COUNT_LAUNCH();
    adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(P, g, m, v, n, lr, b1, b2, eps, scale, bc1, bc2);
}

void launch_propose_hist(const float* logits, long long nb, float logit_thr, unsigned* hist, cudaStream_t st) {
    if (nb <= 0) return;
    GBSDF_COUNT_LAUNCH();
    propose_hist_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(logits, nb, logit_thr, hist);
}

}  // namespace gbsdf
