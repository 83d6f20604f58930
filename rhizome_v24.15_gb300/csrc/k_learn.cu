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

// ---- MLP forward: one thread per sample, BF16 weights staged in shared memory ---------
__global__ void __launch_bounds__(256) mlp_forward_kernel(const float* __restrict__ P, const float* __restrict__ X,
                                                          long long B, float* __restrict__ logits) {
    __shared__ __nv_bfloat16 sW1[kH * kF], sW2[kH * kH], sw3[kH];
    __shared__ float sb1[kH], sb2[kH], sb3;
    for (int i = threadIdx.x; i < kH * kF; i += blockDim.x) sW1[i] = __float2bfloat16_rn(P[oW1 + i]);
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) sW2[i] = __float2bfloat16_rn(P[oW2 + i]);
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        sw3[i] = __float2bfloat16_rn(P[ow3 + i]);
        sb1[i] = P[ob1 + i];
        sb2[i] = P[ob2 + i];
    }
    if (threadIdx.x == 0) sb3 = P[ob3];
    __syncthreads();
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    float x[kF];
    for (int i = 0; i < kF; ++i) x[i] = bf(X[s * kF + i]);
    float h1[kH];
    for (int j = 0; j < kH; ++j) {
        float a = 0.0f;
        for (int i = 0; i < kF; ++i) a = __fmaf_rn(__bfloat162float(sW1[j * kF + i]), x[i], a);
        h1[j] = bf(fmaxf(a + sb1[j], 0.0f));
    }
    float out = 0.0f;
    for (int j = 0; j < kH; ++j) {
        float a = 0.0f;
        for (int i = 0; i < kH; ++i) a = __fmaf_rn(__bfloat162float(sW2[j * kH + i]), h1[i], a);
        const float h2 = bf(fmaxf(a + sb2[j], 0.0f));
        out = __fmaf_rn(__bfloat162float(sw3[j]), h2, out);
    }
    logits[s] = out + sb3;
}

// ---- MLP backward: weighted binary cross-entropy with logits ---------------------------
// Each CTA accumulates the gradient of its samples in shared memory (per-thread rows,
// reduced in a fixed order) and writes one partial; mlp_reduce_kernel sums the partials in
// CTA order, so gradients are deterministic.
constexpr int kBwdThreads = 128;
__global__ void __launch_bounds__(kBwdThreads) mlp_backward_kernel(const float* __restrict__ P,
                                                                   const float* __restrict__ X,
                                                                   const float* __restrict__ y,
                                                                   const float* __restrict__ wt, long long B,
                                                                   float* __restrict__ partial,
                                                                   float* __restrict__ loss_partial) {
    __shared__ __nv_bfloat16 sW1[kH * kF], sW2[kH * kH], sw3[kH];
    __shared__ float sb1[kH], sb2[kH], sb3;
    __shared__ float acc[kMlpParams];
    __shared__ float lred[kBwdThreads];
    for (int i = threadIdx.x; i < kH * kF; i += blockDim.x) sW1[i] = __float2bfloat16_rn(P[oW1 + i]);
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) sW2[i] = __float2bfloat16_rn(P[oW2 + i]);
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        sw3[i] = __float2bfloat16_rn(P[ow3 + i]);
        sb1[i] = P[ob1 + i];
        sb2[i] = P[ob2 + i];
    }
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) acc[i] = 0.0f;
    if (threadIdx.x == 0) sb3 = P[ob3];
    __syncthreads();
    float loss = 0.0f;
    // samples of this CTA, processed one sample per iteration by the whole CTA:
    // thread j < 64 owns hidden unit j, which keeps every accumulation order fixed.
    const long long first = (long long)blockIdx.x * kMlpBwdSamples;
    const long long last = min(B, first + kMlpBwdSamples);
    __shared__ float sx[kF], sh1[kH], sh2[kH], sd2[kH];
    __shared__ float sdl;
    for (long long s = first; s < last; ++s) {
        const int j = threadIdx.x;
        if (j < kF) sx[j] = bf(X[s * kF + j]);
        __syncthreads();
        if (j < kH) {
            float a = 0.0f;
            for (int i = 0; i < kF; ++i) a = __fmaf_rn(__bfloat162float(sW1[j * kF + i]), sx[i], a);
            sh1[j] = a + sb1[j];  // pre-activation
        }
        __syncthreads();
        if (j < kH) {
            float a = 0.0f;
            for (int i = 0; i < kH; ++i) a = __fmaf_rn(__bfloat162float(sW2[j * kH + i]), bf(fmaxf(sh1[i], 0.0f)), a);
            sh2[j] = a + sb2[j];
        }
        __syncthreads();
        if (j == 0) {
            float z = sb3;
            for (int i = 0; i < kH; ++i) z = __fmaf_rn(__bfloat162float(sw3[i]), bf(fmaxf(sh2[i], 0.0f)), z);
            const float yy = y[s], ww = wt ? wt[s] : 1.0f;
            // BCE with logits: w * (max(z,0) - z*y + log(1 + exp(-|z|)))
            loss += ww * (fmaxf(z, 0.0f) - z * yy + log1pf(expf(-fabsf(z))));
            const float p = 1.0f / (1.0f + expf(-z));
            sdl = ww * (p - yy);
            acc[ob3] += sdl;
        }
        __syncthreads();
        if (j < kH) {
            const float a2 = bf(fmaxf(sh2[j], 0.0f));
            acc[ow3 + j] += sdl * a2;
            const float d2 = (sh2[j] > 0.0f) ? sdl * __bfloat162float(sw3[j]) : 0.0f;
            sd2[j] = d2;
            acc[ob2 + j] += d2;
            for (int i = 0; i < kH; ++i) acc[oW2 + j * kH + i] += d2 * bf(fmaxf(sh1[i], 0.0f));
        }
        __syncthreads();
        if (j < kH) {
            float d1 = 0.0f;
            for (int i = 0; i < kH; ++i) d1 = __fmaf_rn(__bfloat162float(sW2[i * kH + j]), sd2[i], d1);
            d1 = (sh1[j] > 0.0f) ? d1 : 0.0f;
            acc[ob1 + j] += d1;
            for (int i = 0; i < kF; ++i) acc[oW1 + j * kF + i] += d1 * sx[i];
        }
        __syncthreads();
    }
    lred[threadIdx.x] = (threadIdx.x == 0) ? loss : 0.0f;
    __syncthreads();
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) partial[(long long)blockIdx.x * kMlpParams + i] = acc[i];
    if (threadIdx.x == 0) loss_partial[blockIdx.x] = lred[0];
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
    GBSDF_COUNT_LAUNCH();
    mlp_forward_kernel<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(P, X, B, logits);
}

int mlp_backward_parts(long long B) { return (int)((B + kMlpBwdSamples - 1) / kMlpBwdSamples); }

void launch_mlp_backward(const float* P, const float* X, const float* y, const float* wt, long long B, float* partial,
                         float* loss_partial, float* grad, float* loss, cudaStream_t st) {
    const int parts = mlp_backward_parts(B);
    if (parts <= 0) return;
    GBSDF_COUNT_LAUNCH();
    mlp_backward_kernel<<<parts, kBwdThreads, 0, st>>>(P, X, y, wt, B, partial, loss_partial);
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
