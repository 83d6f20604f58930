// tune.cu — the sweep-schedule autotuner.
//
// The x sweep has three schedules with identical results (internal header, XSchedule).
// Which one is fastest depends on the lattice (row length, number of CTAs per wave) and
// the device, so the first build of a lattice class times each candidate on that build's
// own buffers -- the band field about to be swept, one warm-up and two timed launches
// each, CUDA events on the build's stream -- and remembers the winner for the class.
// A class is (device, row pitch a multiple of 16 bytes, round(log2 voxels), round(log2
// row length)). Timing writes only the destination copy and one change-flag slot, both
// rewritten by the eikonal stage that follows.
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

using Key = std::tuple<int, int, int, int>;
std::mutex g_tune_mu;
std::map<Key, int> g_tuned;

Key key_of(int device, const Lattice& L) {
    return Key{device, (L.dims[0] & 3) == 0 ? 1 : 0, (int)std::lround(std::log2((double)L.N)),
               (int)std::lround(std::log2((double)L.dims[0]))};
}

}  // namespace

int tuned_x_schedule(int device, const Lattice& L, const float* src, float* dst, const GridMap* src_map,
                     DevState* ds, cudaStream_t st, bool measure) {
    const bool tma = src_map && src_map->valid;
    if (!tma) return kXCpAsync;
    const Key k = key_of(device, L);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tuned.find(k);
        if (it != g_tuned.end()) return it->second;
    }
    if (!measure) return kXTmaPipe;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) {
        cudaGetLastError();
        return kXTmaPipe;
    }
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaGetLastError();
        cudaEventDestroy(a);
        return kXTmaPipe;
    }
    int best = kXTmaPipe;
    float best_ms = 1e30f;
    const int slot = 63;  // a change-flag slot the reference round loop never uses
    for (int cand : {kXCpAsync, kXTmaRing, kXTmaPipe}) {
        launch_sweep(0, 0, 1, slot, src, dst, L, ds, st, src_map, cand);
        cudaEventRecord(a, st);
        for (int r = 0; r < 2; ++r) launch_sweep(0, 0, 1, slot, src, dst, L, ds, st, src_map, cand);
        cudaEventRecord(b, st);
        float ms = 1e30f;
        if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (ms < best_ms) {
            best_ms = ms;
            best = cand;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tuned[k] = best;
    return best;
}

}  // namespace gbsdf
