// noalloc.cu — the exact (legacy-kernel) mesh-to-SDF build without any allocation.
//
// Who needs it: callers that must not call cudaMalloc -- a renderer or simulation step
// that runs under a fixed device-memory budget set at start-up, a plugin running
// inside a host application that owns every device allocation, or a latency-critical
// loop where cudaMalloc's implicit device synchronisation is not acceptable. They
// pass device pointers for the triangles and the output grid; every other buffer this
// build needs (per-tile bounds, 1-bit signs, the FP64 re-check list and the counters)
// lives in one file-scope __device__ array of fixed size, g_noalloc, reserved when the
// library's module is loaded and held by every GPU that loads it until the process
// exits.
//
// Limits (checked before any work; larger inputs are rejected with GBSDF_EINVAL):
//   voxels            <= 16,777,216                (2^24, e.g. 256^3)
//   sign words        <= 1,048,576                 (ceil(dims.x / 32) * dims.y * dims.z)
//   triangles         <= 1,048,576                 (2^20)
// Voxels whose FP32 winding number is close to 0.5 (or has a term of uncertain sign)
// are queued for an FP64 re-check in a list of 1,048,576 entries; past that, a voxel is
// re-checked in FP64 by its own thread. The array is about 12.6 MB.
//
// The computation is the one of gbsdf_compute_mesh_sdf with GBSDF_PATH_LEGACY (the
// reference's mesh_to_sdf_kernel, cuda_rasterizer.cu:97-185, with exact winding signs):
// the squared distances are written straight into the caller's output grid and turned
// into signed distances in place.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gbsdf.h"
#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

constexpr long long kNaMaxVoxels = 1ll << 24;
constexpr long long kNaMaxWords = 1ll << 20;
constexpr long long kNaMaxTris = 1ll << 20;
constexpr long long kNaRecheckCap = 1ll << 20;
constexpr int kNaTile = 128;  // RASTER_TILE_SIZE (math_utils.cuh:35)
constexpr long long kNaMaxTiles = (kNaMaxTris + kNaTile - 1) / kNaTile;

struct NoAllocScratch {
    uint32_t sbits[kNaMaxWords];          // 1-bit inside flags, x fastest, rows padded to 32
    float tile_bounds[kNaMaxTiles * 6];   // per 128-triangle tile: min xyz, max xyz
    long long recheck[kNaRecheckCap];     // voxels decided in FP64
    unsigned long long recheck_n;         // entries written to recheck (may exceed the cap)
    unsigned long long fp64_done;
};

// The scratch array itself. Host code must not use &g_noalloc (that is a host-side
// stand-in); it uses the device address returned by cudaGetSymbolAddress.
static __device__ __align__(256) NoAllocScratch g_noalloc;

constexpr int kNaThreads = 256;

__global__ void na_tile_bounds_kernel(const float* __restrict__ t12, long long T, NoAllocScratch* sc) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ntiles = (T + kNaTile - 1) / kNaTile;
    if (k >= ntiles) return;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (long long i = k * kNaTile; i < min(T, (k + 1) * kNaTile); ++i)
        for (int a = 0; a < 3; ++a) {
            const float v0 = t12[12 * i + a], v1 = t12[12 * i + 3 + a], v2 = t12[12 * i + 6 + a];
            lo[a] = fminf(lo[a], fminf(v0, fminf(v1, v2)));
            hi[a] = fmaxf(hi[a], fmaxf(v0, fmaxf(v1, v2)));
        }
    for (int a = 0; a < 3; ++a) {
        sc->tile_bounds[6 * k + a] = lo[a];
        sc->tile_bounds[6 * k + 3 + a] = hi[a];
    }
}

// Minimum squared distance over all triangles, 128-triangle tiles skipped when their
// box distance is not below the running minimum; written into `out`.
__global__ void __launch_bounds__(kNaThreads) na_dist_kernel(const float* __restrict__ t12, long long T, Lattice L,
                                                             const NoAllocScratch* __restrict__ sc,
                                                             float* __restrict__ out) {
    __shared__ float s[kNaTile * 9];
    const long long ntiles = (T + kNaTile - 1) / kNaTile;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = v < L.N;
    int x = 0, y = 0, z = 0;
    if (ok) {
        x = (int)(v % L.dims[0]);
        const long long r = v / L.dims[0];
        y = (int)(r % L.dims[1]);
        z = (int)(r / L.dims[1]);
    }
    const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, y, z, L.h);
    float mind = 1e12f;
    for (long long t = 0; t < ntiles; ++t) {
        const long long t0 = t * kNaTile;
        const int m = (int)min((long long)kNaTile, T - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < m * 9; k += blockDim.x) {
            const int tri = k / 9, c = k - tri * 9;
            s[k] = t12[(t0 + tri) * 12 + c];
        }
        __syncthreads();
        if (!ok) continue;
        const float* hh = sc->tile_bounds + 6 * t;
        const float bdx = (p.x < hh[0]) ? (hh[0] - p.x) : ((p.x > hh[3]) ? (p.x - hh[3]) : 0.0f);
        const float bdy = (p.y < hh[1]) ? (hh[1] - p.y) : ((p.y > hh[4]) ? (p.y - hh[4]) : 0.0f);
        const float bdz = (p.z < hh[2]) ? (hh[2] - p.z) : ((p.z > hh[5]) ? (p.z - hh[5]) : 0.0f);
        const float box = bdx * bdx + bdy * bdy + bdz * bdz;
        if (!(box < mind)) continue;
        for (int i = 0; i < m; ++i) {
            const float* q = s + 9 * i;
            const float d2 = ptd_sq(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
            if (d2 < mind) mind = d2;
        }
    }
    if (ok) out[v] = mind;
}

__device__ __forceinline__ void na_set_inside(NoAllocScratch* sc, const Lattice& L, long long v) {
    const int x = (int)(v % L.dims[0]);
    const long long row = v / L.dims[0];
    atomicOr(&sc->sbits[(size_t)row * L.wx + (x >> 5)], 1u << (x & 31));
}

// Exact winding sign of every voxel: on-surface voxels (|d| <= 1e-5 voxel) inside;
// otherwise a compensated FP32 sum, FP64 re-check when it is near 0.5 or ambiguous.
__global__ void __launch_bounds__(kNaThreads) na_gwn_kernel(const float* __restrict__ t12, long long T, Lattice L,
                                                            const float* __restrict__ d2, NoAllocScratch* sc) {
    __shared__ float s[256 * 9];
    const float tau = kSurfaceTolVoxels * L.h;
    for (long long base = (long long)blockIdx.x * kNaThreads; base < L.N; base += (long long)gridDim.x * kNaThreads) {
        long long v = base + threadIdx.x;
        f3 p = mk(0.f, 0.f, 0.f);
        if (v < L.N) {
            const int x = (int)(v % L.dims[0]);
            const long long r = v / L.dims[0];
            p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, (int)(r % L.dims[1]), (int)(r / L.dims[1]), L.h);
            if (d2[v] <= tau * tau) {
                na_set_inside(sc, L, v);
                v = -1;
            }
        } else {
            v = -1;
        }
        float sum = 0.0f, comp = 0.0f;
        bool amb = false;
        for (long long c0 = 0; c0 < T; c0 += 256) {
            const int m = (int)min(256ll, T - c0);
            __syncthreads();
            for (int k = threadIdx.x; k < m * 9; k += kNaThreads) {
                const int tri = k / 9, c = k - tri * 9;
                s[k] = t12[(c0 + tri) * 12 + c];
            }
            __syncthreads();
            if (v >= 0) {
                for (int i = 0; i < m; ++i) {
                    const float* q = s + 9 * i;
                    const float om =
                        solid_angle_fast(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]), amb);
                    const float yk = om - comp;
                    const float tk = sum + yk;
                    comp = (tk - sum) - yk;
                    sum = tk;
                }
            }
        }
        if (v >= 0) {
            const float aw = fabsf((sum - comp) * kInv4Pi);
            if (amb || fabsf(aw - 0.5f) < kRecheckBand) {
                const unsigned long long r = atomicAdd(&sc->recheck_n, 1ull);
                if ((long long)r < kNaRecheckCap) {
                    sc->recheck[r] = v;
                } else {  // list full: this thread decides in FP64 itself
                    double acc = 0.0;
                    for (long long t = 0; t < T; ++t) {
                        const float* q = t12 + 12 * t;
                        acc += solid_angle_f64(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
                    }
                    if (fabs(acc / (4.0 * 3.14159265358979323846)) >= 0.5) na_set_inside(sc, L, v);
                    atomicAdd(&sc->fp64_done, 1ull);
                }
            } else if (aw >= 0.5f) {
                na_set_inside(sc, L, v);
            }
        }
    }
}

__global__ void __launch_bounds__(256) na_recheck_kernel(const float* __restrict__ t12, long long T, Lattice L,
                                                         NoAllocScratch* sc) {
    __shared__ double red[256];
    const long long n = min((long long)sc->recheck_n, kNaRecheckCap);
    for (long long e = blockIdx.x; e < n; e += gridDim.x) {
        const long long v = sc->recheck[e];
        const int x = (int)(v % L.dims[0]);
        const long long r = v / L.dims[0];
        const f3 p = lattice_point(L.mn[0], L.mn[1], L.mn[2], x, (int)(r % L.dims[1]), (int)(r / L.dims[1]), L.h);
        double acc = 0.0;
        for (long long t = threadIdx.x; t < T; t += 256) {
            const float* q = t12 + 12 * t;
            acc += solid_angle_f64(p, mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), mk(q[6], q[7], q[8]));
        }
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (fabs(red[0] / (4.0 * 3.14159265358979323846)) >= 0.5) na_set_inside(sc, L, v);
            atomicAdd(&sc->fp64_done, 1ull);
        }
        __syncthreads();
    }
}

// out = (inside ? -1 : 1) * sqrt(min d^2), in place (cuda_rasterizer.cu:181-184)
__global__ void na_combine_kernel(float* __restrict__ out, Lattice L, const NoAllocScratch* __restrict__ sc) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.N; i += stride) {
        const long long row = i / L.dims[0];
        const int x = (int)(i - row * L.dims[0]);
        const bool in = (sc->sbits[(size_t)row * L.wx + (x >> 5)] >> (x & 31)) & 1u;
        const float sg = in ? -1.0f : 1.0f;
        out[i] = sg * sqrtf(out[i]);
    }
}

// Device address of g_noalloc, resolved once per device (with that device current).
std::mutex g_na_mu;
NoAllocScratch* g_na_ptr[64] = {};

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_legacy_sdf_noalloc(const gbsdf_tri* tris_dev, int64_t n_tris, float voxel_size,
                                        const int32_t min_coord[3], const int32_t max_coord[3], float* out_dev,
                                        int32_t device, void* stream, gbsdf_stats* stats, char* err,
                                        size_t errlen) {
    auto fail = [&](int status, const char* msg) {
        if (err && errlen) snprintf(err, errlen, "%s", msg);
        if (stats) stats->status = status;
        return status;
    };
    if (err && errlen) err[0] = 0;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->path_taken = GBSDF_PATH_LEGACY;
    }
    if (!tris_dev || !out_dev || !min_coord || !max_coord) return fail(GBSDF_EINVAL, "null pointer argument");
    if (n_tris <= 0) return fail(GBSDF_EINVAL, "no triangles");
    if (!(voxel_size > 0.0f) || !std::isfinite(voxel_size)) return fail(GBSDF_EINVAL, "bad voxel size");
    long long dims[3];
    for (int k = 0; k < 3; ++k) dims[k] = (long long)max_coord[k] - min_coord[k] + 1;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return fail(GBSDF_EINVAL, "empty lattice");
    const long long N = dims[0] * dims[1] * dims[2];
    const long long words = ((dims[0] + 31) / 32) * dims[1] * dims[2];
    char msg[256];
    if (N > kNaMaxVoxels) {
        snprintf(msg, sizeof(msg), "lattice of %lld voxels exceeds the no-allocation limit of %lld", N, kNaMaxVoxels);
        return fail(GBSDF_EINVAL, msg);
    }
    if (words > kNaMaxWords) {
        snprintf(msg, sizeof(msg), "lattice needs %lld sign words, above the no-allocation limit of %lld", words,
                 kNaMaxWords);
        return fail(GBSDF_EINVAL, msg);
    }
    if (n_tris > kNaMaxTris) {
        snprintf(msg, sizeof(msg), "%lld triangles exceed the no-allocation limit of %lld", (long long)n_tris,
                 kNaMaxTris);
        return fail(GBSDF_EINVAL, msg);
    }
    if (device < 0 || device >= 64) return fail(GBSDF_ENODEV, "device out of range");
    std::lock_guard<std::mutex> lk(g_na_mu);  // calls share g_noalloc: one at a time
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return fail(GBSDF_ENODEV, "cannot select the CUDA device");
    }
    if (!g_na_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            cudaSetDevice(cur);
            snprintf(msg, sizeof(msg), "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return fail(GBSDF_ECUDA, msg);
        }
        g_na_ptr[device] = static_cast<NoAllocScratch*>(p);
    }
    NoAllocScratch* sc = g_na_ptr[device];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Lattice L{};
    for (int k = 0; k < 3; ++k) {
        L.mn[k] = min_coord[k];
        L.dims[k] = (int)dims[k];
    }
    L.h = voxel_size;
    L.N = N;
    L.wx = (int)((dims[0] + 31) / 32);
    L.nwords = words;
    L.px = L.dims[0];
    const float* t12 = reinterpret_cast<const float*>(tris_dev);
    const long long T = n_tris;
    const long long ntiles = (T + kNaTile - 1) / kNaTile;
    cudaError_t e = cudaMemsetAsync(sc->sbits, 0, (size_t)words * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(&sc->recheck_n, 0, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        na_tile_bounds_kernel<<<(unsigned)((ntiles + 127) / 128), 128, 0, st>>>(t12, T, sc);
        na_dist_kernel<<<(unsigned)((N + kNaThreads - 1) / kNaThreads), kNaThreads, 0, st>>>(t12, T, L, sc, out_dev);
        na_gwn_kernel<<<152 * 8, kNaThreads, 0, st>>>(t12, T, L, out_dev, sc);
        na_recheck_kernel<<<152 * 4, 256, 0, st>>>(t12, T, L, sc);
        na_combine_kernel<<<(unsigned)std::min<long long>((N + 255) / 256, 152LL * 32), 256, 0, st>>>(out_dev, L, sc);
        e = cudaGetLastError();
    }
    unsigned long long counts[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, &sc->recheck_n, sizeof(counts), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaSetDevice(cur);
    if (e != cudaSuccess) {
        cudaGetLastError();
        snprintf(msg, sizeof(msg), "CUDA error: %s", cudaGetErrorString(e));
        return fail(GBSDF_ECUDA, msg);
    }
    if (stats) {
        stats->status = GBSDF_OK;
        stats->fp64_rechecks = (long long)counts[1];
        stats->gwn_pairs = N * T;
        stats->kernel_launches = 5;
    }
    return GBSDF_OK;
}
