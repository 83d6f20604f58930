// k_orient.cu — the orientation pre-pass of mesh input (consistent winding, outward).
//
// Reference: CudaRasterizer::orient_mesh_gpu (native/src/engine/mesh/cuda_mesh_topology.cu:
// 707-842, kernels :253-455). Its rule, kept here: an edge used by exactly two triangles
// links them, "same direction" when both traverse it the same way (inconsistent winding);
// every connected component takes the orientation of its smallest triangle (flip parity
// along the links); a component whose links contradict each other is non-orientable;
// flips are applied when any link was inconsistent; the whole mesh is inverted when its
// signed volume is below -1e-5.
//
// GB300 form, deterministic and run to convergence:
//   * edges go into an open-addressing table keyed by (min, max) vertex; a slot records
//     the use count and, for the first two uses, the triangle and its direction bit (the
//     link's "same" flag compares the bits, so which use came first does not matter);
//   * each triangle's <= 3 links are sorted by neighbour after the scatter;
//   * labels propagate Jacobi-style (double-buffered): a triangle takes the smallest
//     component label among itself and its links with the parity the link requires; the
//     loop runs until a sweep changes nothing (the reference stops after 256 in-place
//     sweeps, which leaves large meshes partly unoriented and depends on scheduling);
//   * the signed volume is an FP64 sum in a fixed order (per-CTA partials, one CTA
//     reduces them), so the inversion decision does not depend on atomics.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gbsdf.h"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

struct EdgeSlot {
    unsigned long long key;  // (min << 32 | max) + 1, 0 = empty
    unsigned count;
    unsigned tri_a, tri_b;
    unsigned fwd;  // bit 0: first use runs min -> max, bit 1: second use does
};

__device__ __forceinline__ uint32_t mix32(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}

__global__ void orient_edges_kernel(const uint32_t* __restrict__ idx, long long T, EdgeSlot* __restrict__ table,
                                    uint32_t mask) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    for (int e = 0; e < 3; ++e) {
        const uint32_t u = idx[3 * t + e], v = idx[3 * t + (e + 1) % 3];
        if (u == v) continue;
        const uint32_t lo = min(u, v), hi = max(u, v);
        const unsigned long long key = (((unsigned long long)lo << 32) | hi) + 1ull;
        uint32_t h = mix32(key) & mask;
        for (uint32_t probe = 0; probe <= mask; ++probe) {
            const unsigned long long prev = atomicCAS(&table[h].key, 0ull, key);
            if (prev == 0ull || prev == key) {
                const unsigned c = atomicAdd(&table[h].count, 1u);
                const unsigned fwd = (u < v) ? 1u : 0u;
                if (c == 0) {
                    table[h].tri_a = (unsigned)t;
                    atomicOr(&table[h].fwd, fwd);
                } else if (c == 1) {
                    table[h].tri_b = (unsigned)t;
                    atomicOr(&table[h].fwd, fwd << 1);
                }
                break;
            }
            h = (h + 1) & mask;
        }
    }
}

__global__ void orient_links_kernel(const EdgeSlot* __restrict__ table, long long cap, int* __restrict__ adj,
                                    int* __restrict__ same, int* __restrict__ cnt, int* __restrict__ flags) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    const EdgeSlot s = table[i];
    if (s.key == 0ull || s.count != 2u || s.tri_a == s.tri_b) return;
    const int sm = ((s.fwd & 1u) == ((s.fwd >> 1) & 1u)) ? 1 : 0;
    if (sm) flags[1] = 1;
    const int a = (int)s.tri_a, b = (int)s.tri_b;
    const int ka = atomicAdd(&cnt[a], 1), kb = atomicAdd(&cnt[b], 1);
    if (ka < 3) {
        adj[3 * a + ka] = b;
        same[3 * a + ka] = sm;
    }
    if (kb < 3) {
        adj[3 * b + kb] = a;
        same[3 * b + kb] = sm;
    }
}

// sort each triangle's links by neighbour (a fixed order for the propagation's ties)
__global__ void orient_sort_kernel(long long T, int* __restrict__ adj, int* __restrict__ same, int* __restrict__ cnt,
                                   int* __restrict__ comp, int* __restrict__ flip) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int c = min(cnt[t], 3);
    cnt[t] = c;
    int a[3], s[3];
    for (int k = 0; k < c; ++k) {
        a[k] = adj[3 * t + k];
        s[k] = same[3 * t + k];
    }
    for (int i = 1; i < c; ++i)
        for (int j = i; j > 0 && a[j] < a[j - 1]; --j) {
            const int ta = a[j], ts = s[j];
            a[j] = a[j - 1];
            s[j] = s[j - 1];
            a[j - 1] = ta;
            s[j - 1] = ts;
        }
    for (int k = 0; k < c; ++k) {
        adj[3 * t + k] = a[k];
        same[3 * t + k] = s[k];
    }
    comp[t] = (int)t;
    flip[t] = 0;
}

// one Jacobi step: smallest label among self and links, with the parity the link requires
__global__ void orient_step_kernel(long long T, const int* __restrict__ adj, const int* __restrict__ same,
                                   const int* __restrict__ cnt, const int* __restrict__ comp_in,
                                   const int* __restrict__ flip_in, int* __restrict__ comp_out,
                                   int* __restrict__ flip_out, int* __restrict__ changed) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    int c = comp_in[t], f = flip_in[t];
    const int n = cnt[t];
    for (int k = 0; k < n; ++k) {
        const int nb = adj[3 * t + k];
        const int nc = comp_in[nb];
        if (nc < c) {
            c = nc;
            f = flip_in[nb] ^ same[3 * t + k];
        }
    }
    comp_out[t] = c;
    flip_out[t] = f;
    if (c != comp_in[t] || f != flip_in[t]) *changed = 1;
}

// after convergence: a link whose parity disagrees marks the mesh non-orientable
__global__ void orient_check_kernel(long long T, const int* __restrict__ adj, const int* __restrict__ same,
                                    const int* __restrict__ cnt, const int* __restrict__ flip,
                                    int* __restrict__ flags) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    for (int k = 0; k < cnt[t]; ++k)
        if ((flip[adj[3 * t + k]] ^ same[3 * t + k]) != flip[t]) flags[2] = 1;
}

__global__ void orient_apply_kernel(uint32_t* __restrict__ idx, long long T, const int* __restrict__ flip,
                                    const int* __restrict__ flags) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T || !flags[1] || !flip[t]) return;
    const uint32_t a = idx[3 * t + 1];
    idx[3 * t + 1] = idx[3 * t + 2];
    idx[3 * t + 2] = a;
}

constexpr int kVolThreads = 256;
__global__ void __launch_bounds__(kVolThreads) volume_partial_kernel(const float* __restrict__ v,
                                                                     const uint32_t* __restrict__ idx, long long T,
                                                                     double* __restrict__ part) {
    __shared__ double red[kVolThreads];
    double s = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (long long)gridDim.x * blockDim.x) {
        const float* a = v + 3ull * idx[3 * t];
        const float* b = v + 3ull * idx[3 * t + 1];
        const float* c = v + 3ull * idx[3 * t + 2];
        const double cx = (double)b[1] * c[2] - (double)b[2] * c[1];
        const double cy = (double)b[2] * c[0] - (double)b[0] * c[2];
        const double cz = (double)b[0] * c[1] - (double)b[1] * c[0];
        s += (double)a[0] * cx + (double)a[1] * cy + (double)a[2] * cz;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = kVolThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void volume_final_kernel(const double* __restrict__ part, int n, double* __restrict__ vol6) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    *vol6 = s;
}

__global__ void invert_kernel(uint32_t* __restrict__ idx, long long T) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint32_t a = idx[3 * t + 1];
    idx[3 * t + 1] = idx[3 * t + 2];
    idx[3 * t + 2] = a;
}

struct OErr {
    char* buf;
    size_t len;
    int set(int status, const char* fmt, ...) {
        if (buf && len > 0) {
            va_list ap;
            va_start(ap, fmt);
            vsnprintf(buf, len, fmt, ap);
            va_end(ap);
        }
        return status;
    }
};

unsigned nblk(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_orient_mesh(const float* vertices, int64_t n_vertices, uint32_t* indices, int64_t n_indices,
                                 int32_t* is_orientable, int32_t* had_inconsistent_winding, int32_t* was_inverted,
                                 double* signed_volume, int32_t device, char* err, size_t errlen) {
    OErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (is_orientable) *is_orientable = 1;
    if (had_inconsistent_winding) *had_inconsistent_winding = 0;
    if (was_inverted) *was_inverted = 0;
    if (signed_volume) *signed_volume = 0.0;
    const long long T = n_indices / 3;
    if (T <= 0 || n_vertices <= 0) return GBSDF_OK;  // nothing to orient (cuda_mesh_topology.cu:721-724)
    if (!vertices || !indices) return e.set(GBSDF_EINVAL, "null mesh arrays");
    if (T > 0x3fffffffLL) return e.set(GBSDF_EINVAL, "too many triangles");
    for (long long i = 0; i < 3 * T; ++i)
        if ((int64_t)indices[i] >= n_vertices) return e.set(GBSDF_EINVAL, "index %u out of range", indices[i]);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device %d", device);
    }
    cudaSetDevice(device);
    uint32_t cap = 1024;
    while ((long long)cap < 6 * T + 1024) cap <<= 1;
    const int vparts = (int)std::min<long long>(1024, (T + kVolThreads - 1) / kVolThreads);
    std::vector<void*> mem;
    auto get = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
        mem.push_back(p);
        return p;
    };
    auto cleanup = [&]() {
        for (void* p : mem) cudaFree(p);
    };
    float* d_v = (float*)get((size_t)n_vertices * 12);
    uint32_t* d_i = (uint32_t*)get((size_t)T * 12);
    EdgeSlot* d_tab = (EdgeSlot*)get((size_t)cap * sizeof(EdgeSlot));
    int* d_adj = (int*)get((size_t)T * 12);
    int* d_same = (int*)get((size_t)T * 12);
    int* d_cnt = (int*)get((size_t)T * 4);
    int* d_comp[2] = {(int*)get((size_t)T * 4), (int*)get((size_t)T * 4)};
    int* d_flip[2] = {(int*)get((size_t)T * 4), (int*)get((size_t)T * 4)};
    int* d_flags = (int*)get(4 * sizeof(int));  // [0] changed, [1] inconsistent, [2] non-orientable
    double* d_part = (double*)get((size_t)vparts * 8);
    double* d_vol = (double*)get(8);
    if (mem.size() != 13) {
        cudaGetLastError();
        cleanup();
        return e.set(GBSDF_ENOMEM, "device allocation failed");
    }
    cudaStream_t st = 0;
    cudaMemcpyAsync(d_v, vertices, (size_t)n_vertices * 12, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_i, indices, (size_t)T * 12, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_tab, 0, (size_t)cap * sizeof(EdgeSlot), st);
    cudaMemsetAsync(d_cnt, 0, (size_t)T * 4, st);
    cudaMemsetAsync(d_flags, 0, 4 * sizeof(int), st);
    GBSDF_COUNT_LAUNCH();
    orient_edges_kernel<<<nblk(T), 256, 0, st>>>(d_i, T, d_tab, cap - 1);
    GBSDF_COUNT_LAUNCH();
    orient_links_kernel<<<nblk(cap), 256, 0, st>>>(d_tab, cap, d_adj, d_same, d_cnt, d_flags);
    GBSDF_COUNT_LAUNCH();
    orient_sort_kernel<<<nblk(T), 256, 0, st>>>(T, d_adj, d_same, d_cnt, d_comp[0], d_flip[0]);
    // label propagation until a step changes nothing (at most T steps)
    int cur = 0;
    const int kBatch = 16;
    for (long long it = 0; it < T + kBatch; it += kBatch) {
        cudaMemsetAsync(d_flags, 0, sizeof(int), st);
        for (int k = 0; k < kBatch; ++k) {
            GBSDF_COUNT_LAUNCH();
            orient_step_kernel<<<nblk(T), 256, 0, st>>>(T, d_adj, d_same, d_cnt, d_comp[cur], d_flip[cur],
                                                        d_comp[cur ^ 1], d_flip[cur ^ 1], d_flags);
            cur ^= 1;
        }
        int changed = 0;
        if (cudaMemcpy(&changed, d_flags, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) break;
        if (!changed) break;
    }
    GBSDF_COUNT_LAUNCH();
    orient_check_kernel<<<nblk(T), 256, 0, st>>>(T, d_adj, d_same, d_cnt, d_flip[cur], d_flags);
    GBSDF_COUNT_LAUNCH();
    orient_apply_kernel<<<nblk(T), 256, 0, st>>>(d_i, T, d_flip[cur], d_flags);
    GBSDF_COUNT_LAUNCH();
    volume_partial_kernel<<<vparts, kVolThreads, 0, st>>>(d_v, d_i, T, d_part);
    GBSDF_COUNT_LAUNCH();
    volume_final_kernel<<<1, 32, 0, st>>>(d_part, vparts, d_vol);
    int flags[4] = {0, 0, 0, 0};
    double vol6 = 0.0;
    cudaMemcpy(flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost);
    cudaError_t ce = cudaMemcpy(&vol6, d_vol, 8, cudaMemcpyDeviceToHost);
    double vol = vol6 / 6.0;
    const bool invert = vol < -1e-5;
    if (ce == cudaSuccess && invert) {
        GBSDF_COUNT_LAUNCH();
        invert_kernel<<<nblk(T), 256, 0, st>>>(d_i, T);
        vol = -vol;
    }
    if (ce == cudaSuccess && (flags[1] || invert)) ce = cudaMemcpy(indices, d_i, (size_t)T * 12, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    cleanup();
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "orientation pass: %s", cudaGetErrorString(ce));
    if (is_orientable) *is_orientable = flags[2] ? 0 : 1;
    if (had_inconsistent_winding) *had_inconsistent_winding = flags[1] ? 1 : 0;
    if (was_inverted) *was_inverted = invert ? 1 : 0;
    if (signed_volume) *signed_volume = vol;
    return GBSDF_OK;
}
