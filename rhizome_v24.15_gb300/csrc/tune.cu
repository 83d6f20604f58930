// tune.cu — the autotuner: sweep schedules, and the band splat's tile cut per lattice class.
//
// The x sweep has five schedules and the y / z walks four, all with identical results
// (internal header, XSchedule / WSchedule). Which is fastest depends on the lattice (row
// length, CTAs per wave), the device and the field: the first round sweeps a band in a far
// field, where most updates are one-dimensional, later rounds a field where most warps
// need the 2D and 3D updates. The first build of a lattice class times each candidate on
// that build's own buffers on the field after the first round (phase 1) -- one warm-up and
// two timed launches each (x sweeps for the x schedules, z walks for the walk schedules),
// CUDA events on the build's stream -- and remembers the winners for the later rounds. The
// first round (phase 0) runs the default plan: timed on the band field alone the
// candidates' order did not hold over the round. A caller may still ask for a measured
// phase-0 plan (measure = true with phase 0). A class is (device, row pitch a multiple of 16
// bytes, round(log2 voxels), round(log2 row length)). Timing writes only the destination
// copy, which the next sweep rewrites whole, and one change-flag slot.
//
// The band splat takes a brick either whole in one CTA (splat_kernel) or as eight 4^3
// sub-bricks, one warp each, behind a per-sub-brick triangle bound (splat_dense_kernel);
// the cut between them (binned triangles per brick) is tuned per class of (device,
// round(log2 voxels), round(log2 triangles)) by the engine's first build of the class,
// which times the splat stage at each candidate cut (same results at every cut).
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

using Key = std::tuple<int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<Key, SweepPlan> g_tuned;

Key key_of(int device, const Lattice& L, int phase) {
    return Key{device, (L.px & 3) == 0 ? 1 : 0, (int)std::lround(std::log2((double)L.N)),
               (int)std::lround(std::log2((double)L.dims[0])), phase};
}

}  // namespace

namespace {
using CutKey = std::tuple<int, int, int>;
std::map<CutKey, unsigned> g_cuts;
CutKey cut_key(int device, const Lattice& L, long long T) {
    return CutKey{device, (int)std::lround(std::log2((double)L.N)),
                  (int)std::lround(std::log2((double)std::max(T, 1LL)))};
}
}  // namespace

unsigned tuned_dense_cut(int device, const Lattice& L, long long T) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_cuts.find(cut_key(device, L, T));
    return it == g_cuts.end() ? 0u : it->second;
}

void set_tuned_dense_cut(int device, const Lattice& L, long long T, unsigned cut) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_cuts[cut_key(device, L, T)] = cut;
}

SweepPlan tuned_sweep_plan(int device, const Lattice& L, const float* src, float* dst, const GridMap* src_map,
                           DevState* ds, cudaStream_t st, bool measure, int phase) {
    SweepPlan plan{kXCpAsync, kWCpAsync};
    const bool tma = src_map && src_map->valid, wtma = src_map && src_map->walk_valid;
    if (!tma && !wtma) return plan;
    const Key k = key_of(device, L, phase);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tuned.find(k);
        if (it != g_tuned.end()) return it->second;
    }
    plan = SweepPlan{tma ? kXTmaPipe : kXCpAsync, wtma ? kWTmaVec2 : kWCpAsync};
    if (!measure) return plan;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) {
        cudaGetLastError();
        return plan;
    }
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaGetLastError();
        cudaEventDestroy(a);
        return plan;
    }
    const int slot = 63;  // a change-flag slot the reference round loop never uses
    // one warm-up and two timed launches of one directional sweep; < 0 on failure
    auto time_it = [&](int axis, int xs, int ws) -> float {
        launch_sweep(0, axis, 1, slot, src, dst, L, ds, st, src_map, xs, ws);
        cudaEventRecord(a, st);
        for (int r = 0; r < 2; ++r) launch_sweep(0, axis, 1, slot, src, dst, L, ds, st, src_map, xs, ws);
        cudaEventRecord(b, st);
        float ms = -1.0f;
        if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
            cudaGetLastError();
            return -1.0f;
        }
        return ms;
    };
    if (tma) {
        float best = 1e30f;
        for (int cand : {kXCpAsync, kXTmaRing, kXTmaPipe, kXTmaPipe2, kXTmaWide}) {
            const float ms = time_it(0, cand, plan.w);
            if (ms >= 0.0f && ms < best) {
                best = ms;
                plan.x = cand;
            }
        }
    }
    if (wtma) {
        float best = 1e30f;
        for (int cand : {kWCpAsync, kWTmaPipe, kWTmaVec, kWTmaVec2}) {
            const float ms = time_it(2, plan.x, cand);
            if (ms >= 0.0f && ms < best) {
                best = ms;
                plan.w = cand;
            }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tuned[k] = plan;
    return plan;
}

}  // namespace gbsdf
