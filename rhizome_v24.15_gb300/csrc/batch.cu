// batch.cu — planned batches: many meshes of uneven size built by one CUDA graph.
//
// The single-mesh path (engine.cu) synchronises with the host a few times per build
// (list sizes after binning, the fixup's pass loop, the final status). A planned batch
// removes every one of them from the build itself:
//   * plan: one counting pass (upload, prep, scans) per mesh, one synchronisation, then
//     every buffer of every mesh is carved from one device arena, with the pair lists
//     sized from the counts (plus headroom);
//   * capture: the whole build of each mesh is recorded on its own stream, forked from
//     and joined to one origin stream, into one CUDA graph -- a branch per mesh, so the
//     small meshes' launch-bound stages overlap the large meshes' sweeps. Launch grids
//     that depend on counts read them on the device (splat over the lattice's bricks,
//     persistent exact-winding passes), the fixup runs a fixed number of list passes, and
//     a device-side check decides whether the mesh's output is written;
//   * run: replay the graph, then read each mesh's state once. A run whose counts
//     outgrow the planned lists (new triangle contents) re-plans and runs again.
// Host triangles and host outputs go through pinned staging buffers owned by the batch
// (a graph's copies need page-locked memory, and a failing mesh's output stays untouched).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/gbsdf.h"
#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

struct gbsdf_batch;

namespace gbsdf {
namespace {

constexpr long long kBatchListCap = 8ll * 1024 * 1024;  // same as the single-mesh path
constexpr size_t kAlign = 256;

struct BErr {
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

#define GBB_CK(call)                                                                                    \
    do {                                                                                                \
        cudaError_t _e = (call);                                                                        \
        if (_e != cudaSuccess) {                                                                        \
            cudaGetLastError();                                                                         \
            return e.set(_e == cudaErrorMemoryAllocation ? GBSDF_ENOMEM : GBSDF_ECUDA, "%s: %s (%s:%d)", \
                         #call, cudaGetErrorString(_e), __FILE__, __LINE__);                            \
        }                                                                                               \
    } while (0)

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Job {
    // the caller's mesh
    const float* tris = nullptr;
    long long T = 0;
    float h = 0.0f;
    int32_t mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    float* out = nullptr;
    Lattice L{};
    int pre_status = GBSDF_OK;  // argument checks (the mesh is left out of the graph)
    unsigned dense_cut = kDenseCutDefault;  // the splat's tile cut: the class's tuned value if timed
    // device buffers (offsets into the arenas)
    float *A = nullptr, *B = nullptr, *t12 = nullptr, *t9 = nullptr;
    uint32_t *S = nullptr, *U = nullptr;
    SplatTri* stt = nullptr;
    ParTri* ptt = nullptr;
    unsigned *bcount = nullptr, *bcur = nullptr, *active = nullptr, *scount = nullptr, *scur = nullptr;
    unsigned long long *boff = nullptr, *soff = nullptr, *scan = nullptr;
    long long *list = nullptr, *recheck = nullptr;
    unsigned *blist = nullptr, *slist = nullptr;
    DevState* ds = nullptr;
    long long list_cap = 0;
    unsigned long long cap_b = 0, cap_s = 0;
    // pinned staging and the host mirror of the state
    float* hin = nullptr;
    float* hout = nullptr;
    DevState* hs = nullptr;
    cudaStream_t st = nullptr;
    GridMap map_a{}, map_b{};  // TMA descriptors of A and B
    Fwn fwn{};                 // clusters of the hierarchical winding evaluation
    int xsched = kXAuto;       // sweep schedules of the first round (a tuned class's winners,
    int wsched = kWAuto;       // else the defaults) ...
    int xsched1 = kXAuto;      // ... and of the later rounds
    int wsched1 = kWAuto;
    // learned mode: the signed-crossing pass, the exact-decided mask, the brick features,
    // the open-edge table, the network's logits and the proposal histogram
    uint32_t *S2 = nullptr, *U2 = nullptr, *E = nullptr;
    float *fbase = nullptr, *fX = nullptr, *logits = nullptr;
    unsigned *opencnt = nullptr, *ecnt = nullptr, *phist = nullptr;
    unsigned long long* ekeys = nullptr;
    long long ecap = 0;
};

// Carves aligned sub-buffers out of one allocation: a sizing pass, then a placing pass.
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* take(size_t bytes) {
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += align_up(bytes);
        return p;
    }
};

}  // namespace
}  // namespace gbsdf

struct gbsdf_batch {
    int device = 0;
    int mode = GBSDF_MODE_REFERENCE;
    int num_sms = 0;
    int sweep_schedule = 0;
    int dense_cut = 0;  // gbsdf_options.splat_dense_cut
    bool out_dev = false;
    bool tris_dev = false;
    std::vector<gbsdf::Job> jobs;
    void* arena1 = nullptr;  // everything but the pair lists
    void* arena2 = nullptr;  // the pair lists
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long launches_per_run = 0;
    // learned mode: the network's parameters (device memory, the caller's), the proposal
    // threshold as a logit and the budget (0: 1/16 of each lattice's bricks)
    const float* mlp_params = nullptr;
    float logit_thr = 0.0f;
    unsigned budget = 0;
};

namespace gbsdf {
namespace {

bool exact_signs_mode(const gbsdf_batch& b) { return b.mode == GBSDF_MODE_EXACT_SIGNS; }
bool learned_mode(const gbsdf_batch& b) { return b.mode == GBSDF_MODE_LEARNED; }

void place_learned(Job& j, Carver& c) {
    const Lattice& L = j.L;
    j.S2 = c.take<uint32_t>((size_t)L.nwords * 4);
    j.U2 = c.take<uint32_t>((size_t)L.nwords * 4);
    j.E = c.take<uint32_t>((size_t)L.nwords * 4);
    j.fbase = c.take<float>((size_t)L.nbricks * kBrickBase * 4);
    j.fX = c.take<float>((size_t)L.nbricks * kMlpIn * 4);
    j.logits = c.take<float>((size_t)L.nbricks * 4);
    j.opencnt = c.take<unsigned>((size_t)L.nbricks * 4);
    j.phist = c.take<unsigned>((size_t)kPropBins * 4);
    j.ecap = edge_table_cap(j.T);
    j.ekeys = c.take<unsigned long long>((size_t)j.ecap * 8);
    j.ecnt = c.take<unsigned>((size_t)j.ecap * 4);
}

void place_phase1(Job& j, Carver& c) {
    const Lattice& L = j.L;
    const long long N = L.N, T = j.T;
    // the grid copies also hold the eikonal's padded layout (rows of a multiple of 8 floats)
    j.A = c.take<float>((size_t)std::max(N, padded_voxels(L)) * 4);
    j.B = c.take<float>((size_t)std::max(N, padded_voxels(L)) * 4);
    j.S = c.take<uint32_t>((size_t)L.nwords * 4);
    j.U = c.take<uint32_t>((size_t)L.nwords * 4);
    j.t12 = c.take<float>((size_t)T * 48);
    j.t9 = c.take<float>((size_t)T * 36);
    j.stt = c.take<SplatTri>((size_t)T * sizeof(SplatTri));
    j.ptt = c.take<ParTri>((size_t)T * sizeof(ParTri));
    j.bcount = c.take<unsigned>((size_t)L.nbricks * 4);
    j.bcur = c.take<unsigned>((size_t)L.nbricks * 4);
    j.active = c.take<unsigned>((size_t)L.nbricks * 4);
    j.boff = c.take<unsigned long long>((size_t)L.nbricks * 8);
    j.scount = c.take<unsigned>((size_t)L.nstrips * 4);
    j.scur = c.take<unsigned>((size_t)L.nstrips * 4);
    j.soff = c.take<unsigned long long>((size_t)L.nstrips * 8);
    j.scan = c.take<unsigned long long>((size_t)std::max(scan_tmp_elems(L.nbricks), scan_tmp_elems(L.nstrips)) * 8);
    j.list_cap = std::max<long long>(kVerifySamples, std::min<long long>(kBatchListCap, N));
    j.list = c.take<long long>((size_t)j.list_cap * 8);
    j.recheck = c.take<long long>((size_t)j.list_cap * 8);
    j.ds = c.take<DevState>(sizeof(DevState));
    j.fwn.g = fwn_grid(L, T);
    const long long nc = j.fwn.g.cells;
    const long long ncap = std::max<long long>(1, std::min<long long>(nc, T));
    j.fwn.cells = c.take<FwnCell>((size_t)ncap * sizeof(FwnCell));
    j.fwn.tri = c.take<unsigned>((size_t)T * 4);
    j.fwn.cell_of = c.take<unsigned>((size_t)T * 4);
    j.fwn.counts = c.take<unsigned>((size_t)nc * 4);
    j.fwn.cursor = c.take<unsigned>((size_t)nc * 4);
    j.fwn.flag = c.take<unsigned>((size_t)nc * 4);
    j.fwn.off = c.take<unsigned long long>((size_t)nc * 8);
    j.fwn.cidx = c.take<unsigned long long>((size_t)nc * 8);
    j.fwn.scan = c.take<unsigned long long>((size_t)fwn_scan_elems(j.fwn.g) * 8);
    j.fwn.fb = c.take<long long>((size_t)j.list_cap * 8);
    j.fwn.fb_cap = j.list_cap;
    void* sup = c.take<char>(fwn_super_bytes(j.fwn.g, T, j.list_cap));
    if (sup) fwn_super_carve(j.fwn, sup, T, j.list_cap);
}

void place_phase2(Job& j, Carver& c) {
    j.blist = c.take<unsigned>((size_t)std::max<unsigned long long>(j.cap_b, 1) * 4);
    j.slist = c.take<unsigned>((size_t)std::max<unsigned long long>(j.cap_s, 1) * 4);
}

// Upload + prep + counts (the part of a build whose results size the pair lists).
void enqueue_counts(gbsdf_batch& b, Job& j, cudaStream_t st) {
    const Lattice& L = j.L;
    const long long T = j.T;
    if (b.tris_dev)
        cudaMemcpyAsync(j.t12, j.tris, (size_t)T * 48, cudaMemcpyDeviceToDevice, st);
    else
        cudaMemcpyAsync(j.t12, j.hin, (size_t)T * 48, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(j.ds, 0, sizeof(DevState), st);
    cudaMemsetAsync(j.bcount, 0, (size_t)L.nbricks * 4, st);
    cudaMemsetAsync(j.scount, 0, (size_t)L.nstrips * 4, st);
    launch_prep(j.t12, T, L, j.stt, j.ptt, j.bcount, j.scount, j.ds, st);
    launch_exclusive_scan(j.bcount, j.boff, L.nbricks, j.scan, 0, st);
    launch_exclusive_scan(j.scount, j.soff, L.nstrips, j.scan, 0, st);
    launch_active_bricks(j.bcount, L.nbricks, j.active, j.ds, st, j.dense_cut);
    launch_pack_tri9(j.t12, T, j.t9, st);
}

// The rest of a build, with no host round trip.
void enqueue_build(gbsdf_batch& b, Job& j, cudaStream_t st) {
    const Lattice& L = j.L;
    const long long T = j.T, N = L.N;
    const bool xs = exact_signs_mode(b);
    const float stol = xs ? kSurfaceTolExactSigns : kSurfaceTolVoxels;
    cudaMemsetAsync(j.bcur, 0, (size_t)L.nbricks * 4, st);
    cudaMemsetAsync(j.scur, 0, (size_t)L.nstrips * 4, st);
    launch_bin_fill(j.stt, j.ptt, T, L, j.boff, j.bcur, j.blist, j.soff, j.scur, j.slist, st, j.ds, j.cap_b, j.cap_s);
    launch_fwn_build(j.t9, T, L, j.fwn, j.ds, st);
    // [init] + [A]: one CTA per brick of the lattice, the surplus over the active count exits
    launch_fill(j.A, N, kFarSentinel, st);
    launch_splat(j.stt, j.boff, j.bcount, j.blist, j.active, -1, -1, L, j.A, j.ds, st);
    launch_band_error(j.stt, j.boff, j.bcount, j.blist, L, j.A, j.ds, st);
    // [B]
    launch_parity(j.ptt, j.soff, j.scount, j.slist, L, j.S, j.U, j.ds, xs ? 1 : 0, st);
    // [C]: enough list passes to drain every voxel of the lattice (learned mode records the
    // voxels decided exactly in E, a feature of the sign-risk model)
    const bool learned = learned_mode(b);
    if (learned) cudaMemsetAsync(j.E, 0, (size_t)L.nwords * 4, st);
    const long long passes = std::min<long long>(64, (N + j.list_cap - 1) / j.list_cap + 1);
    auto fixup_passes = [&](uint32_t* ebits) {
        for (long long p = 0; p < passes; ++p) {
            cudaMemsetAsync(&j.ds->listed, 0, sizeof(unsigned long long), st);
            cudaMemsetAsync(&j.ds->list_overflow, 0, sizeof(unsigned long long), st);
            cudaMemsetAsync(&j.ds->recheck_n, 0, sizeof(unsigned long long), st);
            launch_list_unknown(j.U, j.S, L, j.list, j.list_cap, j.ds, 0, st, ebits);
            launch_winding(&j.fwn, j.t9, T, L, j.list, j.list_cap, kGwnFixup, 0, j.S, j.recheck, j.list_cap, j.A, 0,
                           stol, j.ds, b.num_sms, st);
            launch_gwn_recheck(j.t9, T, L, j.recheck, j.list_cap, kGwnFixup, j.S, j.ds, b.num_sms, st);
        }
    };
    fixup_passes(learned ? j.E : nullptr);
    // [D]: the reference's round loop, stopped on the device when a round changes nothing;
    // a lattice whose rows are not a multiple of 8 floats is swept in padded copies (B <->
    // A), the result copied back into A
    const Lattice Lp = padded(L);
    const bool pad = Lp.px != L.dims[0];
    float* src = pad ? j.B : j.A;
    float* dst = pad ? j.A : j.B;
    if (pad) launch_pad_rows(j.A, j.B, Lp, st);
    for (int r = 0; r < kMaxRounds; ++r) {
        for (int axis = 0; axis < 3; ++axis)
            for (int dir = 1; dir >= -1; dir -= 2) {
                launch_sweep(0, axis, dir, r, src, dst, Lp, j.ds, st, src == j.A ? &j.map_a : &j.map_b,
                             r == 0 ? j.xsched : j.xsched1, r == 0 ? j.wsched : j.wsched1);
                std::swap(src, dst);
            }
        launch_end_round(r, r, kMaxRounds, j.ds, st);
    }
    if (pad) launch_unpad_rows(j.B, j.A, Lp, st, j.ds);  // with the audit's count
    else launch_audit(j.A, L, j.ds, st);
    launch_clamp(j.A, j.S, L, j.ds, st);
    // [E]
    for (int gen = 0; gen < kProbeGens; ++gen) {
        launch_verify_prepare(L, gen, j.U, j.list, j.ds, st);
        launch_winding(&j.fwn, j.t9, T, L, j.list, j.list_cap, kGwnVerify, 0, j.S, j.recheck, j.list_cap, j.A, 0,
                       stol, j.ds, b.num_sms, st);
        launch_gwn_recheck(j.t9, T, L, j.recheck, j.list_cap, kGwnVerify, j.S, j.ds, b.num_sms, st);
        launch_verify_plan(gen, j.ds, st, learned ? 1 : 0);
        if (gen == kProbeGens - 1) break;
        launch_patch_mark(L, j.U, j.ds, st);
        launch_list_unknown(j.U, j.S, L, j.list, j.list_cap, j.ds, 1, st, learned ? j.E : nullptr);
        launch_winding(&j.fwn, j.t9, T, L, j.list, j.list_cap, kGwnFixup, 1, j.S, j.recheck, j.list_cap, j.A, 0,
                       stol, j.ds, b.num_sms, st);
        launch_gwn_recheck(j.t9, T, L, j.recheck, j.list_cap, kGwnFixup, j.S, j.ds, b.num_sms, st);
    }
    // learned mode, as in the single-mesh path: the signed-crossing pass (its unknown
    // columns are not counted), escalation of a diverged verify, the brick features, the
    // network's scores and the budgeted proposals, re-decided by the exact winding number
    if (learned) {
        cudaMemcpyAsync(&j.ds->unknown_columns_kept, &j.ds->unknown_columns, 8, cudaMemcpyDeviceToDevice, st);
        launch_parity(j.ptt, j.soff, j.scount, j.slist, L, j.S2, j.U2, j.ds, 1, st);
        cudaMemcpyAsync(&j.ds->unknown_columns, &j.ds->unknown_columns_kept, 8, cudaMemcpyDeviceToDevice, st);
        launch_escalate(j.ds, j.S, j.U, j.S2, j.U2, L, b.num_sms, st);
        fixup_passes(j.E);
        cudaMemsetAsync(j.ekeys, 0, (size_t)j.ecap * 8, st);
        cudaMemsetAsync(j.ecnt, 0, (size_t)j.ecap * 4, st);
        cudaMemsetAsync(j.opencnt, 0, (size_t)L.nbricks * 4, st);
        launch_open_edges(j.t12, T, L, j.ekeys, j.ecnt, j.ecap, j.opencnt, st);
        launch_brick_features(j.A, j.S, j.E, j.S2, j.U2, j.bcount, j.opencnt, L, j.fbase, j.fX, st);
        launch_mlp_forward(b.mlp_params, j.fX, L.nbricks, j.logits, st);
        const unsigned budget = b.budget > 0 ? b.budget : (unsigned)std::max<long long>(1, L.nbricks / 16);
        launch_propose_dev(j.logits, L, b.logit_thr, budget, j.phist, j.ds, j.U, st);
        fixup_passes(nullptr);
    }
    // [F], written only when the build passed its checks
    launch_batch_finalize(j.ds, learned ? 0 : 1, st);
    launch_apply(j.A, j.S, L, b.out_dev ? j.out : j.B, j.ds, xs ? stol * L.h : -1.0f, st);
    if (!b.out_dev) cudaMemcpyAsync(j.hout, j.B, (size_t)N * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(j.hs, j.ds, sizeof(DevState), cudaMemcpyDeviceToHost, st);
}

void free_plan(gbsdf_batch& b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
    if (b.arena1) cudaFree(b.arena1);
    if (b.arena2) cudaFree(b.arena2);
    b.arena1 = b.arena2 = nullptr;
}

// Counts, allocation and graph capture.
int plan(gbsdf_batch& b, BErr& e) {
    free_plan(b);
    // phase 1 buffers
    Carver c1;
    for (Job& j : b.jobs)
        if (j.pre_status == GBSDF_OK) {
            place_phase1(j, c1);
            if (learned_mode(b)) place_learned(j, c1);
        }
    GBB_CK(cudaMalloc(&b.arena1, std::max<size_t>(c1.off, 256)));
    Carver p1{static_cast<char*>(b.arena1), 0};
    for (Job& j : b.jobs)
        if (j.pre_status == GBSDF_OK) {
            place_phase1(j, p1);
            if (learned_mode(b)) place_learned(j, p1);
            const Lattice Lp = padded(j.L);
            encode_grid_map(j.map_a, j.A, Lp);
            encode_grid_map(j.map_b, j.B, Lp);
            const SweepPlan plan = tuned_sweep_plan(b.device, Lp, j.A, j.B, &j.map_a, j.ds, b.origin, false, 0);
            const SweepPlan plan1 = tuned_sweep_plan(b.device, Lp, j.A, j.B, &j.map_a, j.ds, b.origin, false, 1);
            j.xsched = plan.x;
            j.wsched = plan.w;
            if (const unsigned cut = b.dense_cut > 0 ? (unsigned)b.dense_cut : tuned_dense_cut(b.device, j.L, j.T))
                j.dense_cut = cut;
            j.xsched1 = plan1.x;
            j.wsched1 = plan1.w;
            const int xs_opt = b.sweep_schedule % 10, ws_opt = b.sweep_schedule / 10;
            if (xs_opt >= kXCpAsync && xs_opt <= kXTmaWide) j.xsched = j.xsched1 = xs_opt;
            if (ws_opt >= kWCpAsync && ws_opt <= kWTmaVec2) j.wsched = j.wsched1 = ws_opt;
        }
    // counting pass
    for (Job& j : b.jobs) {
        if (j.pre_status != GBSDF_OK) continue;
        if (!b.tris_dev) std::memcpy(j.hin, j.tris, (size_t)j.T * 48);
        enqueue_counts(b, j, b.origin);
        GBB_CK(cudaMemcpyAsync(j.hs, j.ds, sizeof(DevState), cudaMemcpyDeviceToHost, b.origin));
    }
    GBB_CK(cudaGetLastError());
    GBB_CK(cudaStreamSynchronize(b.origin));
    Carver c2;
    for (Job& j : b.jobs) {
        if (j.pre_status != GBSDF_OK) continue;
        // headroom for new triangle contents of the same size
        j.cap_b = j.hs->brick_pairs + j.hs->brick_pairs / 8 + 1024;
        j.cap_s = j.hs->strip_pairs + j.hs->strip_pairs / 8 + 1024;
        place_phase2(j, c2);
    }
    GBB_CK(cudaMalloc(&b.arena2, std::max<size_t>(c2.off, 256)));
    Carver p2{static_cast<char*>(b.arena2), 0};
    for (Job& j : b.jobs)
        if (j.pre_status == GBSDF_OK) place_phase2(j, p2);
    // capture: a branch per mesh, largest first
    std::vector<int> order;
    for (int i = 0; i < (int)b.jobs.size(); ++i)
        if (b.jobs[i].pre_status == GBSDF_OK) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b.jobs[a].L.N > b.jobs[c].L.N; });
    const unsigned long long l0 = launch_counter();
    GBB_CK(cudaStreamBeginCapture(b.origin, cudaStreamCaptureModeRelaxed));
    cudaEventRecord(b.fork, b.origin);
    int k = 0;
    for (int i : order) {
        Job& j = b.jobs[i];
        cudaStreamWaitEvent(j.st, b.fork, 0);
        enqueue_counts(b, j, j.st);
        enqueue_build(b, j, j.st);
        cudaEventRecord(b.joins[k], j.st);
        cudaStreamWaitEvent(b.origin, b.joins[k], 0);
        ++k;
    }
    cudaError_t cap_err = cudaGetLastError();
    cudaError_t end_err = cudaStreamEndCapture(b.origin, &b.graph);
    if (cap_err != cudaSuccess || end_err != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ECUDA, "graph capture failed: %s",
                     cudaGetErrorString(cap_err != cudaSuccess ? cap_err : end_err));
    }
    b.launches_per_run = launch_counter() - l0;
    GBB_CK(cudaGraphInstantiate(&b.exec, b.graph, 0));
    return GBSDF_OK;
}

void parallel_copy(void* dst, const void* src, size_t bytes) {
    const size_t kChunk = 64ull << 20;
    if (bytes <= kChunk) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    const size_t per = (bytes + hw - 1) / hw;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hw; ++t) {
        const size_t a = t * per;
        if (a >= bytes) break;
        const size_t n = std::min(per, bytes - a);
        th.emplace_back([=] { std::memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, n); });
    }
    for (auto& x : th) x.join();
}

int status_of(const gbsdf_batch& b, const Job& j, bool& overflow) {
    overflow = false;
    if (j.pre_status != GBSDF_OK) return j.pre_status;
    const DevState& h = *j.hs;
    if (h.overflow) {
        overflow = true;
        return GBSDF_ECUDA;
    }
    if (h.wait_timeouts) return GBSDF_ECUDA;
    if (h.invalid_tris > 0) return GBSDF_EINVAL;
    if (!learned_mode(b) && (h.csr_entries == 0 || h.csr_entries > 100000000ull)) return GBSDF_ECSR;
    if (h.verify_state != 1) return GBSDF_EVERIFY;
    return GBSDF_OK;
}

void fill_stats(const Job& j, int status, float ms, unsigned long long launches, gbsdf_stats* s) {
    std::memset(s, 0, sizeof(*s));
    s->status = status;
    s->path_taken = GBSDF_PATH_FAST;
    s->ms_total = ms;
    s->kernel_launches = (long long)launches;
    if (j.pre_status != GBSDF_OK) return;
    const DevState& h = *j.hs;
    s->eikonal_rounds = h.rounds + (h.far_residual > 0 ? kMaxExtraRounds : 0);
    s->extra_rounds = h.far_residual > 0 ? kMaxExtraRounds : 0;
    s->probes = h.probes;
    s->sites = h.total_sites;
    s->patch_rounds = h.patch_rounds;
    s->splat_dense_cut = (int32_t)j.dense_cut;
    s->unknown_columns = (long long)h.unknown_columns;
    s->fixup_voxels = (long long)h.fixup_voxels;
    s->patched_voxels = (long long)h.patched_voxels;
    s->fp64_rechecks = (long long)h.fp64_rechecks;
    s->band_voxels = (long long)h.band_voxels;
    s->splat_evals = (long long)h.splat_evals;
    s->gwn_pairs = (long long)h.gwn_pairs;
    s->brick_pairs = (long long)h.brick_pairs;
    s->csr_entries = (long long)h.csr_entries;
    s->winding_certified = (long long)h.fwn_certified;
    s->winding_summed = (long long)h.fwn_fallback_total;
    s->proposed = (long long)h.proposed;
    s->escalated = h.escalated;
    std::memcpy(&s->band_err_fp64, &h.band_err_bits, sizeof(double));
    s->band_err_samples = (long long)h.band_err_n;
    s->sweep_schedule = (j.map_a.valid ? (j.xsched1 == kXAuto ? kXTmaPipe : j.xsched1) : kXCpAsync) +
                        10 * (j.map_a.walk_valid ? (j.wsched1 == kWAuto ? kWTmaPipe : j.wsched1) : kWCpAsync);
}

int run_once(gbsdf_batch& b, bool& any_overflow, float& ms, BErr& e) {
    for (Job& j : b.jobs)
        if (j.pre_status == GBSDF_OK && !b.tris_dev) parallel_copy(j.hin, j.tris, (size_t)j.T * 48);
    GBB_CK(cudaEventRecord(b.t0, b.origin));
    GBB_CK(cudaGraphLaunch(b.exec, b.origin));
    GBB_CK(cudaEventRecord(b.t1, b.origin));
    GBB_CK(cudaStreamSynchronize(b.origin));
    GBB_CK(cudaEventElapsedTime(&ms, b.t0, b.t1));
    any_overflow = false;
    for (Job& j : b.jobs) {
        bool ov = false;
        status_of(b, j, ov);
        any_overflow |= ov;
    }
    return GBSDF_OK;
}

void destroy(gbsdf_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->origin) cudaStreamSynchronize(b->origin);
    free_plan(*b);
    for (gbsdf::Job& j : b->jobs) {
        if (j.hin) cudaFreeHost(j.hin);
        if (j.hout) cudaFreeHost(j.hout);
        if (j.hs) cudaFreeHost(j.hs);
        if (j.st) cudaStreamDestroy(j.st);
    }
    for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

int check_member(const gbsdf_mesh_desc& m, int mode, BErr& e) {
    if (!m.tris || m.n_tris <= 0) return e.set(GBSDF_EINVAL, "no triangles");
    if (m.n_tris > 0x7fffffffLL) return e.set(GBSDF_EINVAL, "too many triangles");
    if (!m.out) return e.set(GBSDF_EINVAL, "null output pointer");
    if (!(m.voxel_size > 0.0f) || !std::isfinite(m.voxel_size))
        return e.set(GBSDF_EINVAL, "voxel size must be positive and finite");
    long long d[3];
    for (int k = 0; k < 3; ++k) {
        d[k] = (long long)m.max_coord[k] - m.min_coord[k] + 1;
        if (d[k] <= 0 || d[k] > (1 << 30)) return e.set(GBSDF_EINVAL, "empty or oversized lattice");
    }
    // the reference's int-range guards (cuda_rasterizer.cu:816-820), reference mode only
    // (the engine indexes in 64 bits; exact-signs batches serve such lattices)
    const long long G = 2000000000LL, N = d[0] * d[1] * d[2];
    if (mode == GBSDF_MODE_REFERENCE &&
        (N > G || m.n_tris * d[2] > G || d[0] * d[1] > G || d[0] * d[2] > G || d[1] * d[2] > G))
        return e.set(GBSDF_EGUARD, "reference int-range guard declines the fast path");
    return GBSDF_OK;
}

}  // namespace
}  // namespace gbsdf

using gbsdf::BErr;

extern "C" {

int gbsdf_batch_create(const gbsdf_mesh_desc* meshes, int32_t n_meshes, int32_t out_on_device,
                       const gbsdf_options* opt, gbsdf_batch** batch, char* err, size_t errlen) {
    BErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!batch) return e.set(GBSDF_EINVAL, "null batch pointer");
    *batch = nullptr;
    if (!meshes || n_meshes <= 0) return e.set(GBSDF_EINVAL, "empty batch");
    gbsdf_options o;
    gbsdf_default_options(&o);
    if (opt) o = *opt;
    if (o.mode != GBSDF_MODE_REFERENCE && o.mode != GBSDF_MODE_EXACT_SIGNS && o.mode != GBSDF_MODE_LEARNED)
        return e.set(GBSDF_EINVAL, "planned batches run the reference, exact-signs or learned mode");
    if (o.mode == GBSDF_MODE_LEARNED && !o.mlp_params)
        return e.set(GBSDF_EINVAL, "a learned batch needs mlp_params (device memory)");
    if (o.path == GBSDF_PATH_LEGACY) return e.set(GBSDF_EINVAL, "planned batches run the fast path");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device available");
    }
    if (o.device < 0 || o.device >= ndev) return e.set(GBSDF_ENODEV, "device %d out of range", o.device);
    GBB_CK(cudaSetDevice(o.device));
    gbsdf_batch* b = new gbsdf_batch();
    b->device = o.device;
    b->mode = o.mode;
    b->sweep_schedule = o.sweep_schedule;
    b->dense_cut = o.splat_dense_cut;
    if (o.mode == GBSDF_MODE_LEARNED) {
        const float pthr = (o.mlp_threshold > 0.0f && o.mlp_threshold < 1.0f) ? o.mlp_threshold : 0.5f;
        b->mlp_params = o.mlp_params;
        b->logit_thr = logf(pthr / (1.0f - pthr));
        b->budget = o.mlp_budget > 0 ? (unsigned)o.mlp_budget : 0u;
    }
    b->out_dev = out_on_device != 0;
    b->tris_dev = o.tris_on_device != 0;
    auto fail = [&](int rc) {
        gbsdf::destroy(b);
        return rc;
    };
    if (cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, o.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
        cudaGetLastError();
        return fail(e.set(GBSDF_ECUDA, "stream / event creation failed"));
    }
    b->jobs.resize(n_meshes);
    char one[256];
    for (int i = 0; i < n_meshes; ++i) {
        const gbsdf_mesh_desc& m = meshes[i];
        gbsdf::Job& j = b->jobs[i];
        BErr ei{one, sizeof(one)};
        j.pre_status = gbsdf::check_member(m, o.mode, ei);
        j.tris = reinterpret_cast<const float*>(m.tris);
        j.T = m.n_tris;
        j.h = m.voxel_size;
        j.out = m.out;
        for (int k = 0; k < 3; ++k) {
            j.mn[k] = m.min_coord[k];
            j.mx[k] = m.max_coord[k];
        }
        if (j.pre_status != GBSDF_OK) continue;
        j.L = gbsdf::make_lattice(j.mn, j.mx, j.h);
        if (cudaStreamCreateWithFlags(&j.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void**>(&j.hs), sizeof(gbsdf::DevState), cudaHostAllocDefault) !=
                cudaSuccess ||
            (!b->tris_dev &&
             cudaHostAlloc(reinterpret_cast<void**>(&j.hin), (size_t)j.T * 48, cudaHostAllocDefault) != cudaSuccess) ||
            (!b->out_dev && cudaHostAlloc(reinterpret_cast<void**>(&j.hout), (size_t)j.L.N * 4,
                                          cudaHostAllocDefault) != cudaSuccess)) {
            cudaGetLastError();
            return fail(e.set(GBSDF_ENOMEM, "mesh %d: pinned staging allocation failed", i));
        }
        std::memset(j.hs, 0, sizeof(gbsdf::DevState));
    }
    b->joins.resize(n_meshes);
    for (auto& ev : b->joins)
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return fail(e.set(GBSDF_ECUDA, "event creation failed"));
        }
    int rc = gbsdf::plan(*b, e);
    if (rc != GBSDF_OK) return fail(rc);
    *batch = b;
    return GBSDF_OK;
}

int gbsdf_batch_run(gbsdf_batch* b, int32_t* statuses, gbsdf_stats* stats, char* err, size_t errlen) {
    BErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!b) return e.set(GBSDF_EINVAL, "null batch");
    GBB_CK(cudaSetDevice(b->device));
    bool overflow = false;
    float ms = 0.0f;
    int rc = gbsdf::run_once(*b, overflow, ms, e);
    if (rc != GBSDF_OK) return rc;
    if (overflow) {  // new contents outgrew the planned lists: plan again, run again
        rc = gbsdf::plan(*b, e);
        if (rc != GBSDF_OK) return rc;
        rc = gbsdf::run_once(*b, overflow, ms, e);
        if (rc != GBSDF_OK) return rc;
        if (overflow) return e.set(GBSDF_ECUDA, "batch lists overflowed after re-planning");
    }
    int first = GBSDF_OK;
    for (size_t i = 0; i < b->jobs.size(); ++i) {
        gbsdf::Job& j = b->jobs[i];
        bool ov = false;
        const int s = gbsdf::status_of(*b, j, ov);
        if (s == GBSDF_OK && !b->out_dev) gbsdf::parallel_copy(j.out, j.hout, (size_t)j.L.N * 4);
        if (statuses) statuses[i] = s;
        if (stats) gbsdf::fill_stats(j, s, ms, i == 0 ? b->launches_per_run : 0, &stats[i]);
        if (s != GBSDF_OK && first == GBSDF_OK) {
            first = s;
            e.set(s, "mesh %zu failed with status %d", i, s);
        }
    }
    return first;
}

void gbsdf_batch_destroy(gbsdf_batch* b) { gbsdf::destroy(b); }

}  // extern "C"
