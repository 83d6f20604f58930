// engine.cu — host orchestration and C ABI of the GB300 mesh-to-SDF engine.
//
// One call runs the whole path on one GPU, on one CUDA stream of a per-device
// workspace whose buffers persist across calls (the reference allocates and frees
// every buffer per call, cuda_rasterizer.cu:884-918 and :1141):
//
//   H2D triangles -> [prep] per-triangle records, brick / strip counts
//   -> [bin] counting-sort lists  -> [init] sentinel fill -> [A] brick splat
//   -> [B] parity ballots -> [C] exact winding of unknown columns
//   -> [D] eikonal sweeps (+ audit / clamp) -> [E] stratified verify + patch boxes
//   -> [F] sign apply -> D2H (host output) .
//
// Host synchronisation points: one after binning (list sizes, guards), one after
// the parity pass (unknown-voxel count), one at the end (status); the eikonal round
// loop and the verify / patch loop are driven by device-side state.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gbsdf.h"
#include "gbsdf_device.cuh"
#include "gbsdf_internal.h"

namespace gbsdf {

unsigned long long& launch_counter() {
    static thread_local unsigned long long n = 0;
    return n;
}

Lattice make_lattice(const int32_t mn[3], const int32_t mx[3], float h) {
    Lattice L{};
    for (int k = 0; k < 3; ++k) {
        L.mn[k] = mn[k];
        L.dims[k] = mx[k] - mn[k] + 1;
    }
    L.h = h;
    L.N = (long long)L.dims[0] * L.dims[1] * L.dims[2];
    L.wx = (L.dims[0] + 31) / 32;
    L.nwords = (long long)L.wx * L.dims[1] * L.dims[2];
    for (int k = 0; k < 3; ++k) L.nb[k] = (L.dims[k] + kBrick - 1) / kBrick;
    L.nbricks = (long long)L.nb[0] * L.nb[1] * L.nb[2];
    L.nsx = (L.dims[0] + kStrip - 1) / kStrip;
    L.nstrips = (long long)L.nsx * L.dims[1];
    L.px = L.dims[0];
    return L;
}

namespace {

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Workspace {
    int device = -1;
    int num_sms = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[14] = {};
    std::mutex mu;
    Buf A, B, S, U, t12, t9, stt, ptt, bcount, bcur, boff, active, blist, scount, scur, soff, slist, scan, list,
        recheck, hb, verts, idx, flags, fpos, S2, U2, fbase, fX, logits, opencnt, ekeys, ecnt, mparts, mlossp, phist, E, fwc, fwt, fwo, fwn, fwu, fwf, fwoff,
        fwci, fwscan, fwfb, fws;
    DevState* ds = nullptr;
    DevState* hs = nullptr;  // pinned host mirror
};

Workspace g_ws[64];
std::mutex g_ws_mu;

struct Err {
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

#define GB_CK(call)                                                                                     \
    do {                                                                                                \
        cudaError_t _e = (call);                                                                        \
        if (_e != cudaSuccess) {                                                                        \
            return e.set(_e == cudaErrorMemoryAllocation ? GBSDF_ENOMEM : GBSDF_ECUDA, "%s: %s (%s:%d)", \
                         #call, cudaGetErrorString(_e), __FILE__, __LINE__);                            \
        }                                                                                               \
    } while (0)

cudaError_t ensure(Buf& b, size_t bytes) {
    if (bytes <= b.bytes && b.p) return cudaSuccess;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t err = cudaMalloc(&b.p, want);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return err;
    }
    b.bytes = want;
    return cudaSuccess;
}

template <class T>
T* P(Buf& b) {
    return static_cast<T*>(b.p);
}

// Creates the workspace's stream, events and device-state buffers on `device`. On a
// failure part-way the handles created so far are released again, so a retry starts
// clean and nothing leaks.
int init_ws(Workspace& w, int device, Err& e) {
    if (w.device == device) return GBSDF_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device available");
    }
    if (device < 0 || device >= n) return e.set(GBSDF_ENODEV, "device %d out of range (%d devices)", device, n);
    auto undo = [&w]() {
        for (auto& ev : w.ev) {
            if (ev) cudaEventDestroy(ev);
            ev = nullptr;
        }
        if (w.st) cudaStreamDestroy(w.st);
        if (w.ds) cudaFree(w.ds);
        if (w.hs) cudaFreeHost(w.hs);
        w.st = nullptr;
        w.ds = nullptr;
        w.hs = nullptr;
    };
    cudaError_t err = cudaSetDevice(device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&w.num_sms, cudaDevAttrMultiProcessorCount, device);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&w.st, cudaStreamNonBlocking);
    for (auto& ev : w.ev)
        if (err == cudaSuccess) err = cudaEventCreate(&ev);
    if (err == cudaSuccess) err = cudaMalloc(&w.ds, sizeof(DevState));
    if (err == cudaSuccess) err = cudaMallocHost(&w.hs, sizeof(DevState));
    if (err != cudaSuccess) {
        cudaGetLastError();
        undo();
        return e.set(err == cudaErrorMemoryAllocation ? GBSDF_ENOMEM : GBSDF_ECUDA, "workspace set-up on device %d: %s",
                     device, cudaGetErrorString(err));
    }
    w.device = device;
    return GBSDF_OK;
}

void free_ws(Workspace& w) {
    if (w.device < 0) return;
    cudaSetDevice(w.device);
    Buf* bufs[] = {&w.A, &w.B, &w.S, &w.U, &w.t12, &w.t9, &w.stt, &w.ptt, &w.bcount, &w.bcur, &w.boff,
                   &w.active, &w.blist, &w.scount, &w.scur, &w.soff, &w.slist, &w.scan, &w.list, &w.recheck,
                   &w.hb, &w.verts, &w.idx, &w.flags, &w.fpos, &w.S2, &w.U2, &w.fbase, &w.fX, &w.logits,
                   &w.opencnt, &w.ekeys, &w.ecnt, &w.mparts, &w.mlossp, &w.phist, &w.E,
                   &w.fwc, &w.fwt, &w.fwo, &w.fwn, &w.fwu, &w.fwf, &w.fwoff, &w.fwci, &w.fwscan, &w.fwfb, &w.fws};
    for (Buf* b : bufs) {
        if (b->p) cudaFree(b->p);
        *b = Buf{};
    }
    if (w.ds) cudaFree(w.ds);
    if (w.hs) cudaFreeHost(w.hs);
    for (auto& ev : w.ev)
        if (ev) cudaEventDestroy(ev);
    if (w.st) cudaStreamDestroy(w.st);
    w.ds = nullptr;
    w.hs = nullptr;
    w.st = nullptr;
    for (auto& ev : w.ev) ev = nullptr;
    w.device = -1;
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.0f;
    }
    return ms;
}

constexpr long long kListCap = 8ll * 1024 * 1024;  // >= 64 patch boxes of 49^3 voxels

// Exact winding of every voxel flagged in U (initial unknown columns): compaction
// into the dense list, FP32 pass, FP64 re-checks; repeats while the list overflowed.
// Clusters of the hierarchical winding evaluation for the packed triangles (w.t9).
int build_fwn(Workspace& w, const Lattice& L, long long T, Fwn& f, Err& e) {
    cudaStream_t st = w.st;
    const FwnGrid g = fwn_grid(L, T);
    const long long ncap = std::max<long long>(1, std::min<long long>(g.cells, T));
    GB_CK(ensure(w.fwc, (size_t)ncap * sizeof(FwnCell)));
    GB_CK(ensure(w.fwt, (size_t)T * 4));
    GB_CK(ensure(w.fwo, (size_t)T * 4));
    GB_CK(ensure(w.fwn, (size_t)g.cells * 4));
    GB_CK(ensure(w.fwu, (size_t)g.cells * 4));
    GB_CK(ensure(w.fwf, (size_t)g.cells * 4));
    GB_CK(ensure(w.fwoff, (size_t)g.cells * 8));
    GB_CK(ensure(w.fwci, (size_t)g.cells * 8));
    GB_CK(ensure(w.fwscan, (size_t)fwn_scan_elems(g) * 8));
    GB_CK(ensure(w.fwfb, (size_t)kListCap * 8));
    f = Fwn{g, P<FwnCell>(w.fwc), P<unsigned>(w.fwt), P<unsigned>(w.fwo), P<unsigned>(w.fwn), P<unsigned>(w.fwu),
            P<unsigned>(w.fwf), P<unsigned long long>(w.fwoff), P<unsigned long long>(w.fwci),
            P<unsigned long long>(w.fwscan), P<long long>(w.fwfb), kListCap};
    GB_CK(ensure(w.fws, fwn_super_bytes(g, T, kListCap)));
    fwn_super_carve(f, w.fws.p, T, kListCap);
    launch_fwn_build(P<float>(w.t9), T, L, f, w.ds, st);
    GB_CK(cudaGetLastError());
    return GBSDF_OK;
}

int fixup_unknown(Workspace& w, const Lattice& L, long long T, float stol, Err& e, uint32_t* ebits = nullptr,
                  const Fwn* fwn = nullptr) {
    cudaStream_t st = w.st;
    for (int pass = 0; pass < 1 << 20; ++pass) {
        GB_CK(cudaMemsetAsync(&w.ds->listed, 0, sizeof(unsigned long long), st));
        GB_CK(cudaMemsetAsync(&w.ds->list_overflow, 0, sizeof(unsigned long long), st));
        GB_CK(cudaMemsetAsync(&w.ds->recheck_n, 0, sizeof(unsigned long long), st));
        launch_list_unknown(P<uint32_t>(w.U), P<uint32_t>(w.S), L, P<long long>(w.list), kListCap, w.ds, 0, st,
                            ebits);
        GB_CK(cudaMemcpyAsync(w.hs, w.ds, sizeof(DevState), cudaMemcpyDeviceToHost, st));
        GB_CK(cudaStreamSynchronize(st));
        long long n = std::min<long long>((long long)w.hs->listed, kListCap);
        if (n <= 0) return GBSDF_OK;
        if (fwn)
            launch_winding(fwn, P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnFixup, 0, P<uint32_t>(w.S),
                           P<long long>(w.recheck), kListCap, P<float>(w.A), 0, stol, w.ds, w.num_sms, st);
        else if (n < 64 * 1024)
            launch_gwn_small(P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnFixup, P<uint32_t>(w.S),
                             P<long long>(w.recheck), kListCap, P<float>(w.A), 0, stol, w.ds, n, st);
        else
            launch_gwn(P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnFixup, 0, P<uint32_t>(w.S),
                       P<long long>(w.recheck), kListCap, P<float>(w.A), 0, stol, w.ds, w.num_sms, st);
        launch_gwn_recheck(P<float>(w.t9), T, L, P<long long>(w.recheck), kListCap, kGwnFixup, P<uint32_t>(w.S),
                           w.ds, w.num_sms, st);
        GB_CK(cudaGetLastError());
        if (w.hs->list_overflow == 0) return GBSDF_OK;
    }
    return e.set(GBSDF_ECUDA, "unknown-voxel fixup did not drain");
}

// The signed-crossing parity pass into w.S2 / w.U2 (learned mode: the escalation's signs
// and a feature input). It adds its unknown columns to the state's count; the reference
// pass's count is kept.
int signed_pass(Workspace& w, const Lattice& L, Err& e) {
    cudaStream_t st = w.st;
    GB_CK(ensure(w.S2, (size_t)L.nwords * 4));
    GB_CK(ensure(w.U2, (size_t)L.nwords * 4));
    GB_CK(cudaMemcpyAsync(&w.hs->unknown_columns, &w.ds->unknown_columns, 8, cudaMemcpyDeviceToHost, st));
    GB_CK(cudaStreamSynchronize(st));
    const unsigned long long unk_ref = w.hs->unknown_columns;
    launch_parity(P<ParTri>(w.ptt), P<unsigned long long>(w.soff), P<unsigned>(w.scount), P<unsigned>(w.slist), L,
                  P<uint32_t>(w.S2), P<uint32_t>(w.U2), w.ds, 1, st);
    GB_CK(cudaMemcpyAsync(&w.ds->unknown_columns, &unk_ref, 8, cudaMemcpyHostToDevice, st));
    GB_CK(cudaGetLastError());
    return GBSDF_OK;
}

// Learned-model brick features into w.fX, from the unsigned distance field (w.A), the
// current signs (w.S), the exact-decided mask (w.E) and the signed-crossing pass
// (w.S2 / w.U2, signed_pass).
int brick_features(Workspace& w, long long T, const Lattice& L, Err& e) {
    cudaStream_t st = w.st;
    GB_CK(ensure(w.fbase, (size_t)L.nbricks * kBrickBase * 4));
    GB_CK(ensure(w.fX, (size_t)L.nbricks * kMlpIn * 4));
    GB_CK(ensure(w.opencnt, (size_t)L.nbricks * 4));
    const long long cap = edge_table_cap(T);
    GB_CK(ensure(w.ekeys, (size_t)cap * 8));
    GB_CK(ensure(w.ecnt, (size_t)cap * 4));
    GB_CK(cudaMemsetAsync(w.ekeys.p, 0, (size_t)cap * 8, st));
    GB_CK(cudaMemsetAsync(w.ecnt.p, 0, (size_t)cap * 4, st));
    GB_CK(cudaMemsetAsync(w.opencnt.p, 0, (size_t)L.nbricks * 4, st));
    launch_open_edges(P<float>(w.t12), T, L, P<unsigned long long>(w.ekeys), P<unsigned>(w.ecnt), cap,
                      P<unsigned>(w.opencnt), st);
    launch_brick_features(P<float>(w.A), P<uint32_t>(w.S), P<uint32_t>(w.E), P<uint32_t>(w.S2), P<uint32_t>(w.U2),
                          P<unsigned>(w.bcount), P<unsigned>(w.opencnt), L, P<float>(w.fbase), P<float>(w.fX), st);
    GB_CK(cudaGetLastError());
    return GBSDF_OK;
}

int run_fast(Workspace& w, long long T, const Lattice& L, const gbsdf_options& o, float* out, bool out_dev,
             gbsdf_stats* stats, Err& e, float* features_out = nullptr) {
    cudaStream_t st = w.st;
    const bool ref_mode = (o.mode == GBSDF_MODE_REFERENCE);
    const bool exact_signs = (o.mode == GBSDF_MODE_EXACT || o.mode == GBSDF_MODE_EXACT_SIGNS);
    const bool ref_eikonal = (o.mode != GBSDF_MODE_EXACT);
    const float stol = exact_signs ? kSurfaceTolExactSigns : kSurfaceTolVoxels;
    const long long N = L.N;
    // ---- buffers
    // the grid copies also hold the eikonal's padded layout (rows of a multiple of 8 floats)
    GB_CK(ensure(w.A, (size_t)std::max(N, padded_voxels(L)) * 4));
    GB_CK(ensure(w.B, (size_t)std::max(N, padded_voxels(L)) * 4));
    GB_CK(ensure(w.S, (size_t)L.nwords * 4));
    GB_CK(ensure(w.U, (size_t)L.nwords * 4));
    GB_CK(ensure(w.t9, (size_t)T * 36));
    GB_CK(ensure(w.stt, (size_t)T * sizeof(SplatTri)));
    GB_CK(ensure(w.ptt, (size_t)T * sizeof(ParTri)));
    GB_CK(ensure(w.bcount, (size_t)L.nbricks * 4));
    GB_CK(ensure(w.bcur, (size_t)L.nbricks * 4));
    GB_CK(ensure(w.boff, (size_t)L.nbricks * 8));
    GB_CK(ensure(w.active, (size_t)L.nbricks * 4));
    GB_CK(ensure(w.scount, (size_t)L.nstrips * 4));
    GB_CK(ensure(w.scur, (size_t)L.nstrips * 4));
    GB_CK(ensure(w.soff, (size_t)L.nstrips * 8));
    GB_CK(ensure(w.scan, (size_t)std::max(scan_tmp_elems(L.nbricks), scan_tmp_elems(L.nstrips)) * 8));
    GB_CK(ensure(w.list, (size_t)kListCap * 8));
    GB_CK(ensure(w.recheck, (size_t)kListCap * 8));

    // ---- [prep] + counts
    GB_CK(cudaMemsetAsync(w.ds, 0, sizeof(DevState), st));
    if (o.wait_poll_limit != 0) {
        w.hs->wait_polls = o.wait_poll_limit;
        GB_CK(cudaMemcpyAsync(&w.ds->wait_polls, &w.hs->wait_polls, sizeof(int), cudaMemcpyHostToDevice, st));
        GB_CK(cudaStreamSynchronize(st));
    }
    GB_CK(cudaMemsetAsync(w.bcount.p, 0, (size_t)L.nbricks * 4, st));
    GB_CK(cudaMemsetAsync(w.scount.p, 0, (size_t)L.nstrips * 4, st));
    launch_prep(P<float>(w.t12), T, L, P<SplatTri>(w.stt), P<ParTri>(w.ptt), P<unsigned>(w.bcount),
                P<unsigned>(w.scount), w.ds, st);
    launch_exclusive_scan(P<unsigned>(w.bcount), P<unsigned long long>(w.boff), L.nbricks,
                          P<unsigned long long>(w.scan), 0, st);
    launch_exclusive_scan(P<unsigned>(w.scount), P<unsigned long long>(w.soff), L.nstrips,
                          P<unsigned long long>(w.scan), 0, st);
    // the splat's tile cut: the class's tuned value, else the default (and timed below)
    const unsigned cut_known = o.splat_dense_cut > 0 ? (unsigned)o.splat_dense_cut : tuned_dense_cut(w.device, L, T);
    unsigned dense_cut = cut_known ? cut_known : kDenseCutDefault;
    launch_active_bricks(P<unsigned>(w.bcount), L.nbricks, P<unsigned>(w.active), w.ds, st, dense_cut);
    launch_pack_tri9(P<float>(w.t12), T, P<float>(w.t9), st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaMemcpyAsync(w.hs, w.ds, sizeof(DevState), cudaMemcpyDeviceToHost, st));
    GB_CK(cudaStreamSynchronize(st));
    if (w.hs->invalid_tris > 0)
        return e.set(GBSDF_EINVAL, "%llu triangles have non-finite or out-of-range coordinates",
                     (unsigned long long)w.hs->invalid_tris);
    if ((ref_mode || o.mode == GBSDF_MODE_EXACT_SIGNS) &&
        (w.hs->csr_entries == 0 || w.hs->csr_entries > 100000000ull))
        return e.set(GBSDF_ECSR, "supercell CSR has %llu entries (reference guard: 1..1e8)",
                     (unsigned long long)w.hs->csr_entries);
    const long long brick_pairs = (long long)w.hs->brick_pairs;
    const long long strip_pairs = (long long)w.hs->strip_pairs;
    long long n_active = (long long)w.hs->active_bricks;
    long long n_dense = (long long)w.hs->dense_bricks;
    GB_CK(ensure(w.blist, (size_t)std::max<long long>(brick_pairs, 1) * 4));
    GB_CK(ensure(w.slist, (size_t)std::max<long long>(strip_pairs, 1) * 4));
    Fwn fwn_s{};
    const Fwn* fwn = nullptr;
    if (o.winding_eval == 0) {
        int rcw = build_fwn(w, L, T, fwn_s, e);
        if (rcw != GBSDF_OK) return rcw;
        fwn = &fwn_s;
    }
    GB_CK(cudaMemsetAsync(w.bcur.p, 0, (size_t)L.nbricks * 4, st));
    GB_CK(cudaMemsetAsync(w.scur.p, 0, (size_t)L.nstrips * 4, st));
    launch_bin_fill(P<SplatTri>(w.stt), P<ParTri>(w.ptt), T, L, P<unsigned long long>(w.boff), P<unsigned>(w.bcur),
                    P<unsigned>(w.blist), P<unsigned long long>(w.soff), P<unsigned>(w.scur), P<unsigned>(w.slist),
                    st);
    if (!cut_known && o.sweep_schedule == 0) {
        // the class's first autotuned build: time the splat stage at each candidate cut on
        // this build's own lists (identical results at every cut), keep the fastest
        auto split = [&](unsigned cut) -> int {
            GB_CK(cudaMemsetAsync(&w.ds->active_bricks, 0, 2 * sizeof(unsigned long long), st));
            launch_active_bricks(P<unsigned>(w.bcount), L.nbricks, P<unsigned>(w.active), w.ds, st, cut);
            GB_CK(cudaMemcpyAsync(&w.hs->active_bricks, &w.ds->active_bricks, 2 * sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, st));
            GB_CK(cudaStreamSynchronize(st));
            n_active = (long long)w.hs->active_bricks;
            n_dense = (long long)w.hs->dense_bricks;
            return (int)GBSDF_OK;
        };
        float best_ms = 1e30f;
        unsigned best = dense_cut;
        for (unsigned cut : {128u, 256u, 512u, 1024u}) {
            if (int rcs = split(cut)) return rcs;
            launch_fill(P<float>(w.A), N, kFarSentinel, st);
            GB_CK(cudaEventRecord(w.ev[10], st));  // events 10 and 11: the tuner's own
            launch_splat(P<SplatTri>(w.stt), P<unsigned long long>(w.boff), P<unsigned>(w.bcount),
                         P<unsigned>(w.blist), P<unsigned>(w.active), n_active, n_dense, L, P<float>(w.A), w.ds, st);
            GB_CK(cudaEventRecord(w.ev[11], st));
            GB_CK(cudaEventSynchronize(w.ev[11]));
            float ms = 0.0f;
            GB_CK(cudaEventElapsedTime(&ms, w.ev[10], w.ev[11]));
            if (ms < best_ms) {
                best_ms = ms;
                best = cut;
            }
        }
        set_tuned_dense_cut(w.device, L, T, best);
        dense_cut = best;
        if (int rcs = split(best)) return rcs;
        // the timed splats counted into the build's statistics: start them again
        GB_CK(cudaMemsetAsync(&w.ds->band_voxels, 0, sizeof(unsigned long long), st));
        GB_CK(cudaMemsetAsync(&w.ds->splat_evals, 0, sizeof(unsigned long long), st));
    }
    GB_CK(cudaEventRecord(w.ev[2], st));
    // ---- [init] + [A]
    launch_fill(P<float>(w.A), N, kFarSentinel, st);
    launch_splat(P<SplatTri>(w.stt), P<unsigned long long>(w.boff), P<unsigned>(w.bcount), P<unsigned>(w.blist),
                 P<unsigned>(w.active), n_active, n_dense, L, P<float>(w.A), w.ds, st);
    launch_band_error(P<SplatTri>(w.stt), P<unsigned long long>(w.boff), P<unsigned>(w.bcount), P<unsigned>(w.blist), L,
                      P<float>(w.A), w.ds, st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[3], st));
    // ---- [B]
    launch_parity(P<ParTri>(w.ptt), P<unsigned long long>(w.soff), P<unsigned>(w.scount), P<unsigned>(w.slist), L,
                  P<uint32_t>(w.S), P<uint32_t>(w.U), w.ds, exact_signs ? 1 : 0, st);
    GB_CK(cudaGetLastError());
    // ---- learned mode: E records every voxel the exact winding number decides, so the
    // brick features (after [E]) can tell the remaining risk apart
    const bool learned = (o.mode == GBSDF_MODE_LEARNED);
    uint32_t* ebits = nullptr;
    if (learned || features_out) {
        GB_CK(ensure(w.E, (size_t)L.nwords * 4));
        GB_CK(cudaMemsetAsync(w.E.p, 0, (size_t)L.nwords * 4, st));
        ebits = P<uint32_t>(w.E);
    }
    GB_CK(cudaEventRecord(w.ev[4], st));
    // ---- [C]
    int rc = fixup_unknown(w, L, T, stol, e, ebits, fwn);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaEventRecord(w.ev[5], st));
    // ---- [D]
    const int rule = ref_eikonal ? 0 : 1;
    // The sweeps address rows of a multiple of 8 floats (padded(L)): a lattice whose rows are
    // not is swept in padded copies. Where the band field's own rows are 16-byte multiples and
    // the first x sweep reads its source through a TMA descriptor, that sweep reads A through a
    // descriptor of A's dense rows and writes the padded copy into B; the rounds ping-pong
    // B <-> A, and the result (back in A, padded) is copied dense into B, which then takes A's
    // place. Otherwise the band field is first copied into B, the rounds ping-pong B <-> A and
    // the result is copied back into A.
    const Lattice Lp = padded(L);
    const bool pad = Lp.px != L.dims[0];
    GridMap map_a, map_b, map_dense;
    encode_grid_map(map_a, P<float>(w.A), Lp);
    encode_grid_map(map_b, P<float>(w.B), Lp);
    const bool dense_map = pad && encode_grid_map(map_dense, P<float>(w.A), L);
    auto map_of = [&](const float* p) { return p == P<float>(w.A) ? &map_a : &map_b; };
    float* src = P<float>(w.A);
    float* dst = P<float>(w.B);
    // sweep_schedule: 0 autotuned; else x schedule + 10 x walk schedule (a 0 digit: tuned).
    // The first round runs the default plan (phase 0, not measured: timed on the band field
    // alone, before any sweep has filled the far field, the candidates' order did not hold
    // for the round, and on the 860 x 860 x 880 mug some builds picked a plan 0.9 ms slower);
    // the later rounds run the plan tuned on the field after the first round (phase 1).
    const int xs_opt = o.sweep_schedule % 10, ws_opt = o.sweep_schedule / 10;
    const bool tune = xs_opt == 0 || ws_opt == 0;
    SweepPlan plan;
    auto set_plan = [&](int phase, const GridMap* m, bool measure) -> int {
        plan = tuned_sweep_plan(w.device, Lp, src, dst, m, w.ds, st, measure, phase);
        if (xs_opt >= kXCpAsync && xs_opt <= kXTmaWide) plan.x = xs_opt;
        if (ws_opt >= kWCpAsync && ws_opt <= kWTmaVec2) plan.w = ws_opt;
        GB_CK(cudaGetLastError());
        return (int)GBSDF_OK;
    };
    if (int rcp = set_plan(0, dense_map ? &map_dense : map_of(src), false)) return rcp;
    const SweepPlan plan0 = plan;
    const bool fused_pad = dense_map && plan.x != kXCpAsync;
    if (pad && !fused_pad) {
        launch_pad_rows(P<float>(w.A), P<float>(w.B), Lp, st);
        std::swap(src, dst);
    }
    const GridMap* lead = fused_pad ? &map_dense : nullptr;  // the first sweep's source descriptor
    GB_CK(cudaEventRecord(w.ev[12], st));  // events 12 and 13: the directional sweeps alone
    if (ref_eikonal) {
        for (int r = 0; r < kMaxRounds; ++r) {
            if (r == 1)
                if (int rcp = set_plan(1, map_of(src), tune)) return rcp;
            for (int axis = 0; axis < 3; ++axis)
                for (int dir = 1; dir >= -1; dir -= 2) {
                    launch_sweep(rule, axis, dir, r, src, dst, Lp, w.ds, st, lead ? lead : map_of(src), plan.x,
                                 plan.w);
                    lead = nullptr;
                    std::swap(src, dst);
                }
            launch_end_round(r, r, kMaxRounds, w.ds, st);
        }
    } else {
        const int cap = o.max_rounds > 0 ? o.max_rounds : 4096;
        const int batch = 4;
        for (int r0 = 0; r0 < cap; r0 += batch) {
            for (int r = r0; r < std::min(cap, r0 + batch); ++r) {
                if (r == 1)
                    if (int rcp = set_plan(1, map_of(src), tune)) return rcp;
                GB_CK(cudaMemsetAsync(&w.ds->changed[r % 64], 0, sizeof(int), st));
                for (int axis = 0; axis < 3; ++axis)
                    for (int dir = 1; dir >= -1; dir -= 2) {
                        launch_sweep(rule, axis, dir, r % 64, src, dst, Lp, w.ds, st, lead ? lead : map_of(src),
                                     plan.x, plan.w);
                        lead = nullptr;
                        std::swap(src, dst);
                    }
                launch_end_round(r % 64, r, cap, w.ds, st);
            }
            GB_CK(cudaMemcpyAsync(&w.hs->stop, &w.ds->stop, sizeof(int), cudaMemcpyDeviceToHost, st));
            GB_CK(cudaStreamSynchronize(st));
            if (w.hs->stop) break;
        }
    }
    GB_CK(cudaEventRecord(w.ev[13], st));
    // rounds are whole (6 sweeps, an even number), so the field is back in the first source
    // (the copy back also takes the audit's count of voxels still at the far sentinel)
    if (fused_pad) {
        launch_unpad_rows(P<float>(w.A), P<float>(w.B), Lp, st, w.ds);
        std::swap(w.A, w.B);  // equal sizes; the field is in A again from here on
    } else if (pad) {
        launch_unpad_rows(P<float>(w.B), P<float>(w.A), Lp, st, w.ds);
    } else {
        launch_audit(P<float>(w.A), L, w.ds, st);
    }
    launch_clamp(P<float>(w.A), P<uint32_t>(w.S), L, w.ds, st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[6], st));
    // ---- [E]
    for (int gen = 0; gen < kProbeGens; ++gen) {
        launch_verify_prepare(L, gen, P<uint32_t>(w.U), P<long long>(w.list), w.ds, st);
        launch_winding(fwn, P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnVerify, 0, P<uint32_t>(w.S),
                       P<long long>(w.recheck), kListCap, P<float>(w.A), 0, stol, w.ds, w.num_sms, st);
        launch_gwn_recheck(P<float>(w.t9), T, L, P<long long>(w.recheck), kListCap, kGwnVerify, P<uint32_t>(w.S),
                           w.ds, w.num_sms, st);
        launch_verify_plan(gen, w.ds, st, learned ? 1 : 0);
        if (gen == kProbeGens - 1) break;  // the last generation never patches
        launch_patch_mark(L, P<uint32_t>(w.U), w.ds, st);
        launch_list_unknown(P<uint32_t>(w.U), P<uint32_t>(w.S), L, P<long long>(w.list), kListCap, w.ds, 1, st,
                            ebits);
        launch_winding(fwn, P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnFixup, 1, P<uint32_t>(w.S),
                       P<long long>(w.recheck), kListCap, P<float>(w.A), 0, stol, w.ds, w.num_sms, st);
        launch_gwn_recheck(P<float>(w.t9), T, L, P<long long>(w.recheck), kListCap, kGwnFixup, P<uint32_t>(w.S),
                           w.ds, w.num_sms, st);
    }
    GB_CK(cudaGetLastError());
    // ---- learned mode, after [E] (the probes and patch boxes ran exactly as in the plain
    // path): the signed-crossing pass; a diverged verify escalates to its signs, its columns
    // through holes decided by the exact winding number, instead of declining; then the
    // brick features, the network's scores and the riskiest bricks re-decided by the exact
    // winding number. The network never supplies a sign.
    if (learned || features_out) {
        int rcs = signed_pass(w, L, e);
        if (rcs != GBSDF_OK) return rcs;
        if (learned) {
            launch_escalate(w.ds, P<uint32_t>(w.S), P<uint32_t>(w.U), P<uint32_t>(w.S2), P<uint32_t>(w.U2), L,
                            w.num_sms, st);
            GB_CK(cudaGetLastError());
            int rce = fixup_unknown(w, L, T, stol, e, ebits, fwn);
            if (rce != GBSDF_OK) return rce;
        }
        int rcf = brick_features(w, T, L, e);
        if (rcf != GBSDF_OK) return rcf;
        if (features_out) {
            GB_CK(cudaMemcpyAsync(features_out, w.fX.p, (size_t)L.nbricks * kMlpIn * 4, cudaMemcpyDeviceToDevice, st));
            GB_CK(cudaStreamSynchronize(st));
            return GBSDF_OK;
        }
        if (!o.mlp_params && !o.brick_scores) return e.set(GBSDF_EINVAL, "learned mode needs mlp_params");
        const float* logits = o.brick_scores;
        if (!logits) {
            GB_CK(ensure(w.logits, (size_t)L.nbricks * 4));
            launch_mlp_forward(o.mlp_params, P<float>(w.fX), L.nbricks, P<float>(w.logits), st);
            logits = P<float>(w.logits);
        }
        const float pthr = (o.mlp_threshold > 0.0f && o.mlp_threshold < 1.0f) ? o.mlp_threshold : 0.5f;
        const float lthr = logf(pthr / (1.0f - pthr));
        const unsigned budget =
            o.mlp_budget > 0 ? (unsigned)o.mlp_budget : (unsigned)std::max<long long>(1, L.nbricks / 16);
        GB_CK(ensure(w.phist, (size_t)kPropBins * 4));
        launch_propose_dev(logits, L, lthr, budget, P<unsigned>(w.phist), w.ds, P<uint32_t>(w.U), st);
        GB_CK(cudaGetLastError());
        int rcp = fixup_unknown(w, L, T, stol, e, nullptr, fwn);
        if (rcp != GBSDF_OK) return rcp;
    }
    GB_CK(cudaEventRecord(w.ev[7], st));
    // ---- [F]
    // a pinned (page-locked) host output is written by the apply kernel itself through its
    // device mapping, which streams the grid over the host link without a staging copy
    float* final_dst = out_dev ? out : P<float>(w.B);
    bool direct_host = false;
    if (!out_dev && o.host_output == 0) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
            final_dst = static_cast<float*>(pa.devicePointer);
            direct_host = true;
        } else {
            cudaGetLastError();
        }
    }
    launch_apply(P<float>(w.A), P<uint32_t>(w.S), L, final_dst, w.ds, exact_signs ? stol * L.h : -1.0f, st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[8], st));
    GB_CK(cudaMemcpyAsync(w.hs, w.ds, sizeof(DevState), cudaMemcpyDeviceToHost, st));
    GB_CK(cudaStreamSynchronize(st));
    const DevState& h = *w.hs;
    int status = GBSDF_OK;
    if (h.wait_timeouts) return e.set(GBSDF_ECUDA, "%llu staged-tile waits of the eikonal sweeps timed out",
                                      (unsigned long long)h.wait_timeouts);
    if (h.verify_state != 1) status = e.set(GBSDF_EVERIFY, "sign verification diverged: %d mismatches in probe %d",
                                            h.probe_m, h.probes - 1);
    if (status == GBSDF_OK && !out_dev && !direct_host) {
        GB_CK(cudaMemcpyAsync(out, w.B.p, (size_t)N * 4, cudaMemcpyDeviceToHost, st));
    }
    GB_CK(cudaEventRecord(w.ev[9], st));
    GB_CK(cudaStreamSynchronize(st));
    if (stats) {
        stats->ms_prep = ev_ms(w.ev[1], w.ev[2]);
        stats->ms_splat = ev_ms(w.ev[2], w.ev[3]);
        stats->ms_parity = ev_ms(w.ev[3], w.ev[4]);
        stats->ms_fixup = ev_ms(w.ev[4], w.ev[5]);
        stats->ms_eikonal = ev_ms(w.ev[5], w.ev[6]);
        stats->ms_sweeps = ev_ms(w.ev[12], w.ev[13]);
        stats->ms_verify = ev_ms(w.ev[6], w.ev[7]);
        stats->ms_apply = ev_ms(w.ev[7], w.ev[8]);
        stats->ms_d2h = ev_ms(w.ev[8], w.ev[9]);
        stats->eikonal_rounds = h.rounds;
        stats->far_residual = (long long)h.far_residual;
        stats->safe_clamped = (long long)h.far_residual;
        // the reference runs up to 16 audit-gated extra rounds while a residual remains
        // (cuda_rasterizer.cu:1028-1037); a residual after a full round means no voxel is
        // reachable (empty band), so those rounds cannot change anything and are counted,
        // not run.
        stats->extra_rounds = (ref_eikonal && h.far_residual > 0) ? kMaxExtraRounds : 0;
        if (ref_eikonal) stats->eikonal_rounds += stats->extra_rounds;
        stats->far_residual = 0;
        stats->probes = h.probes;
        stats->sites = h.total_sites;
        stats->patch_rounds = h.patch_rounds;
        stats->splat_dense_cut = (int32_t)dense_cut;
        stats->unknown_columns = (long long)h.unknown_columns;
        stats->fixup_voxels = (long long)h.fixup_voxels;
        stats->patched_voxels = (long long)h.patched_voxels;
        stats->fp64_rechecks = (long long)h.fp64_rechecks;
        stats->band_voxels = (long long)h.band_voxels;
        stats->splat_evals = (long long)h.splat_evals;
        stats->gwn_pairs = (long long)h.gwn_pairs;
        stats->brick_pairs = (long long)h.brick_pairs;
        stats->csr_entries = (long long)h.csr_entries;
        stats->path_taken = GBSDF_PATH_FAST;
        stats->proposed = (long long)h.proposed;
        stats->escalated = h.escalated;
        std::memcpy(&stats->band_err_fp64, &h.band_err_bits, sizeof(double));
        stats->band_err_samples = (long long)h.band_err_n;
        stats->winding_certified = (long long)h.fwn_certified;
        stats->winding_summed = (long long)h.fwn_fallback_total;
        // x schedule + 10 x walk schedule of the last round's sweeps
        auto code = [&](const SweepPlan& p) {
            return (map_a.valid ? (p.x == kXAuto ? kXTmaPipe : p.x) : kXCpAsync) +
                   10 * (map_a.walk_valid ? (p.w == kWAuto ? kWTmaPipe : p.w) : kWCpAsync);
        };
        stats->sweep_schedule = code(plan);
        stats->sweep_schedule_first = code(plan0);
    }
    return status;
}

int run_legacy(Workspace& w, long long T, const Lattice& L, float* out, bool out_dev, gbsdf_stats* stats, Err& e,
               int winding_eval = 0) {
    cudaStream_t st = w.st;
    const long long N = L.N;
    const long long ntiles = (T + 127) / 128;
    GB_CK(ensure(w.A, (size_t)N * 4));
    GB_CK(ensure(w.B, (size_t)N * 4));
    GB_CK(ensure(w.S, (size_t)L.nwords * 4));
    GB_CK(ensure(w.t9, (size_t)T * 36));
    GB_CK(ensure(w.hb, (size_t)ntiles * 24));
    GB_CK(ensure(w.list, (size_t)kListCap * 8));
    GB_CK(ensure(w.recheck, (size_t)kListCap * 8));
    GB_CK(cudaMemsetAsync(w.ds, 0, sizeof(DevState), st));
    GB_CK(cudaMemsetAsync(w.S.p, 0, (size_t)L.nwords * 4, st));
    launch_pack_tri9(P<float>(w.t12), T, P<float>(w.t9), st);
    launch_tile_bounds(P<float>(w.t12), T, P<float>(w.hb), st);
    GB_CK(cudaEventRecord(w.ev[2], st));
    launch_legacy_dist(P<float>(w.t9), T, P<float>(w.hb), L, P<float>(w.A), st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[3], st));
    // exact winding sign of every voxel, in list-sized chunks
    Fwn fwn_s{};
    const Fwn* fwn = nullptr;
    if (winding_eval == 0) {
        int rcw = build_fwn(w, L, T, fwn_s, e);
        if (rcw != GBSDF_OK) return rcw;
        fwn = &fwn_s;
    }
    for (long long v0 = 0; v0 < N; v0 += kListCap) {
        long long n = std::min(kListCap, N - v0);
        launch_iota(P<long long>(w.list), n, v0, st);
        unsigned long long nn = (unsigned long long)n;
        GB_CK(cudaMemcpyAsync(&w.ds->listed, &nn, sizeof(nn), cudaMemcpyHostToDevice, st));
        GB_CK(cudaMemsetAsync(&w.ds->recheck_n, 0, sizeof(unsigned long long), st));
        launch_winding(fwn, P<float>(w.t9), T, L, P<long long>(w.list), kListCap, kGwnFixup, 0, P<uint32_t>(w.S),
                       P<long long>(w.recheck), kListCap, P<float>(w.A), 1, kSurfaceTolVoxels, w.ds, w.num_sms, st);
        launch_gwn_recheck(P<float>(w.t9), T, L, P<long long>(w.recheck), kListCap, kGwnFixup, P<uint32_t>(w.S),
                           w.ds, w.num_sms, st);
        GB_CK(cudaStreamSynchronize(st));  // `nn` lives on the host stack
    }
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[4], st));
    float* final_dst = out_dev ? out : P<float>(w.B);
    launch_legacy_combine(P<float>(w.A), P<uint32_t>(w.S), L, final_dst, st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaEventRecord(w.ev[8], st));
    if (!out_dev) GB_CK(cudaMemcpyAsync(out, w.B.p, (size_t)N * 4, cudaMemcpyDeviceToHost, st));
    GB_CK(cudaEventRecord(w.ev[9], st));
    GB_CK(cudaMemcpyAsync(w.hs, w.ds, sizeof(DevState), cudaMemcpyDeviceToHost, st));
    GB_CK(cudaStreamSynchronize(st));
    if (stats) {
        stats->ms_prep = ev_ms(w.ev[1], w.ev[2]);
        stats->ms_splat = ev_ms(w.ev[2], w.ev[3]);
        stats->ms_fixup = ev_ms(w.ev[3], w.ev[4]);
        stats->ms_apply = ev_ms(w.ev[4], w.ev[8]);
        stats->ms_d2h = ev_ms(w.ev[8], w.ev[9]);
        stats->gwn_pairs = (long long)w.hs->gwn_pairs;
        stats->fp64_rechecks = (long long)w.hs->fp64_rechecks;
        stats->winding_certified = (long long)w.hs->fwn_certified;
        stats->winding_summed = (long long)w.hs->fwn_fallback_total;
        stats->path_taken = GBSDF_PATH_LEGACY;
    }
    return GBSDF_OK;
}

int compute(const float* tris12, long long T, bool tris_dev, float h, const int32_t mn[3], const int32_t mx[3],
            float* out, bool out_dev, const gbsdf_options& o, gbsdf_stats* stats, Err& e) {
    auto t0 = std::chrono::steady_clock::now();
    const unsigned long long launches0 = launch_counter();
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->status = GBSDF_EINVAL;
    }
    if (!mn || !mx || !out) return e.set(GBSDF_EINVAL, "null lattice or output pointer");
    if (!(h > 0.0f) || !std::isfinite(h)) return e.set(GBSDF_EINVAL, "voxel size must be positive and finite");
    long long dims[3];
    for (int k = 0; k < 3; ++k) dims[k] = (long long)mx[k] - mn[k] + 1;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return e.set(GBSDF_EINVAL, "empty lattice");
    if (T <= 0 || !tris12) return e.set(GBSDF_EINVAL, "no triangles");
    if (dims[0] > (1 << 30) || dims[1] > (1 << 30) || dims[2] > (1 << 30))
        return e.set(GBSDF_EINVAL, "lattice dimension out of range");
    const long long N = dims[0] * dims[1] * dims[2];
    int path = o.path;
    if (path == GBSDF_PATH_AUTO) path = ((unsigned long long)N >= kFastMinVoxels) ? GBSDF_PATH_FAST : GBSDF_PATH_LEGACY;
    // the reference's int-range guards (cuda_rasterizer.cu:816-820): reference mode only (the
    // engine indexes in 64 bits; the other modes serve such lattices)
    if (path == GBSDF_PATH_FAST && o.mode == GBSDF_MODE_REFERENCE) {
        const long long G = 2000000000LL;
        if (N > G || T * dims[2] > G || dims[0] * dims[1] > G || dims[0] * dims[2] > G || dims[1] * dims[2] > G) {
            if (o.path != GBSDF_PATH_AUTO)
                return e.set(GBSDF_EGUARD, "reference int-range guard declines the fast path");
            path = GBSDF_PATH_LEGACY;
        }
    }
    if (T > 0x7fffffffLL) return e.set(GBSDF_EINVAL, "too many triangles");
    Workspace* wp;
    {
        std::lock_guard<std::mutex> g(g_ws_mu);
        if (o.device < 0 || o.device >= 64) return e.set(GBSDF_ENODEV, "device %d out of range", o.device);
        wp = &g_ws[o.device];
    }
    Workspace& w = *wp;
    std::lock_guard<std::mutex> lk(w.mu);
    int rc = init_ws(w, o.device, e);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaSetDevice(o.device));
    Lattice L = make_lattice(mn, mx, h);
    GB_CK(cudaEventRecord(w.ev[0], w.st));
    if (tris_dev) {
        GB_CK(ensure(w.t12, (size_t)T * 48));
        GB_CK(cudaMemcpyAsync(w.t12.p, tris12, (size_t)T * 48, cudaMemcpyDeviceToDevice, w.st));
    } else {
        GB_CK(ensure(w.t12, (size_t)T * 48));
        GB_CK(cudaMemcpyAsync(w.t12.p, tris12, (size_t)T * 48, cudaMemcpyHostToDevice, w.st));
    }
    GB_CK(cudaEventRecord(w.ev[1], w.st));
    if (path == GBSDF_PATH_FAST) {
        rc = run_fast(w, T, L, o, out, out_dev, stats, e);
        if (rc == GBSDF_EVERIFY || rc == GBSDF_ECSR) {
            if (o.path == GBSDF_PATH_AUTO)
                rc = run_legacy(w, T, L, out, out_dev, stats, e, o.winding_eval);  // reference fall-through
        }
    } else {
        rc = run_legacy(w, T, L, out, out_dev, stats, e, o.winding_eval);
    }
    if (stats) {
        stats->ms_h2d = ev_ms(w.ev[0], w.ev[1]);
        stats->status = rc;
        stats->kernel_launches = (long long)(launch_counter() - launches0);
        stats->ms_total =
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (rc != GBSDF_OK) {
        // leave the stream clean for the next call
        cudaStreamSynchronize(w.st);
        cudaGetLastError();
    }
    return rc;
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" {

void gbsdf_default_options(gbsdf_options* opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->mode = GBSDF_MODE_REFERENCE;
    opt->path = GBSDF_PATH_AUTO;
}

int gbsdf_compute_mesh_sdf(const gbsdf_tri* tris, int64_t n_tris, float voxel_size, const int32_t min_coord[3],
                           const int32_t max_coord[3], float* out, int32_t out_on_device, const gbsdf_options* opt,
                           gbsdf_stats* stats, char* err, size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    gbsdf_options o;
    gbsdf_default_options(&o);
    if (opt) o = *opt;
    return compute(reinterpret_cast<const float*>(tris), n_tris, o.tris_on_device != 0, voxel_size, min_coord,
                   max_coord, out, out_on_device != 0, o, stats, e);
}

int gbsdf_compute_mesh_sdf_batch(gbsdf_mesh_desc* meshes, int32_t n_meshes, int32_t out_on_device,
                                 const gbsdf_options* opt, gbsdf_stats* stats, char* err, size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!meshes || n_meshes <= 0) return e.set(GBSDF_EINVAL, "empty batch");
    gbsdf_options o;
    gbsdf_default_options(&o);
    if (opt) o = *opt;
    if (o.path == GBSDF_PATH_FAST && (o.mode == GBSDF_MODE_REFERENCE || o.mode == GBSDF_MODE_EXACT_SIGNS ||
                                      (o.mode == GBSDF_MODE_LEARNED && o.mlp_params && !o.brick_scores))) {
        gbsdf_batch* b = nullptr;
        int rc = gbsdf_batch_create(meshes, n_meshes, out_on_device, &o, &b, err, errlen);
        if (rc != GBSDF_OK) return rc;
        std::vector<int32_t> st(n_meshes, GBSDF_ECUDA);
        rc = gbsdf_batch_run(b, st.data(), stats, err, errlen);
        gbsdf_batch_destroy(b);
        for (int32_t i = 0; i < n_meshes; ++i) meshes[i].status = st[i];
        return rc;
    }
    int first_bad = GBSDF_OK;
    char one[256];
    for (int32_t i = 0; i < n_meshes; ++i) {
        gbsdf_mesh_desc& m = meshes[i];
        Err ei{one, sizeof(one)};
        one[0] = 0;
        m.status = compute(reinterpret_cast<const float*>(m.tris), m.n_tris, o.tris_on_device != 0, m.voxel_size,
                           m.min_coord, m.max_coord, m.out, out_on_device != 0, o, stats ? &stats[i] : nullptr, ei);
        if (m.status != GBSDF_OK && first_bad == GBSDF_OK) {
            first_bad = m.status;
            e.set(m.status, "mesh %d: %s", i, one);
        }
    }
    return first_bad;
}

int gbsdf_mesh_lattice(const float* verts, int64_t n_verts, float voxel_size, int32_t min_coord[3],
                       int32_t max_coord[3], char* err, size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!verts || n_verts <= 0) return e.set(GBSDF_EINVAL, "no vertices");
    if (!(voxel_size > 0.0f) || !std::isfinite(voxel_size)) return e.set(GBSDF_EINVAL, "bad voxel size");
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int64_t i = 0; i < n_verts; ++i)
        for (int k = 0; k < 3; ++k) {
            float v = verts[3 * i + k];
            if (!std::isfinite(v)) return e.set(GBSDF_EINVAL, "non-finite vertex %lld", (long long)i);
            lo[k] = std::fmin(lo[k], v);
            hi[k] = std::fmax(hi[k], v);
        }
    // cuda_rasterizer.cu:1358-1372, with the integer range validated in FP64 first
    float pad = voxel_size * 10.0f;
    for (int k = 0; k < 3; ++k) {
        double a = std::floor((double)((lo[k] - pad) / voxel_size));
        double b = std::ceil((double)((hi[k] + pad) / voxel_size));
        if (!(a > -1.0e9 && b < 1.0e9)) return e.set(GBSDF_EINVAL, "lattice out of integer range");
        min_coord[k] = (int32_t)std::floor((lo[k] - pad) / voxel_size);
        max_coord[k] = (int32_t)std::ceil((hi[k] + pad) / voxel_size);
    }
    return GBSDF_OK;
}

int gbsdf_build_from_mesh(const float* verts, int64_t n_verts, const uint32_t* indices, int64_t n_indices,
                          float voxel_size, const int32_t min_coord[3], const int32_t max_coord[3], float* out,
                          int32_t out_on_device, const gbsdf_options* opt, gbsdf_stats* stats, char* err,
                          size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    gbsdf_options o;
    gbsdf_default_options(&o);
    if (opt) o = *opt;
    if (!verts || n_verts <= 0 || !indices || n_indices < 3) return e.set(GBSDF_EINVAL, "empty mesh");
    const long long nt = n_indices / 3;
    Workspace* wp;
    {
        std::lock_guard<std::mutex> g(g_ws_mu);
        if (o.device < 0 || o.device >= 64) return e.set(GBSDF_ENODEV, "device %d out of range", o.device);
        wp = &g_ws[o.device];
    }
    Workspace& w = *wp;
    long long kept = 0;
    float* tris_dev = nullptr;
    {
        std::lock_guard<std::mutex> lk(w.mu);
        int rc = init_ws(w, o.device, e);
        if (rc != GBSDF_OK) return rc;
        GB_CK(cudaSetDevice(o.device));
        cudaStream_t st = w.st;
        GB_CK(ensure(w.verts, (size_t)n_verts * 12));
        GB_CK(ensure(w.idx, (size_t)nt * 12));
        GB_CK(ensure(w.flags, (size_t)nt * 4));
        GB_CK(ensure(w.fpos, (size_t)nt * 8));
        GB_CK(ensure(w.scan, (size_t)scan_tmp_elems(nt) * 8));
        GB_CK(cudaMemcpyAsync(w.verts.p, verts, (size_t)n_verts * 12, cudaMemcpyHostToDevice, st));
        GB_CK(cudaMemcpyAsync(w.idx.p, indices, (size_t)nt * 12, cudaMemcpyHostToDevice, st));
        launch_tri_flags(P<float>(w.verts), n_verts, P<uint32_t>(w.idx), nt, P<unsigned>(w.flags), st);
        launch_exclusive_scan(P<unsigned>(w.flags), P<unsigned long long>(w.fpos), nt,
                              P<unsigned long long>(w.scan), 0, st);
        unsigned long long last_pos = 0;
        unsigned last_flag = 0;
        GB_CK(cudaMemcpyAsync(&last_pos, P<unsigned long long>(w.fpos) + (nt - 1), 8, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaMemcpyAsync(&last_flag, P<unsigned>(w.flags) + (nt - 1), 4, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaStreamSynchronize(st));
        kept = (long long)last_pos + last_flag;
        if (kept <= 0) return e.set(GBSDF_EINVAL, "mesh has no non-degenerate triangle");
        GB_CK(cudaMalloc(&tris_dev, (size_t)kept * 48));
        launch_tri_scatter(P<float>(w.verts), n_verts, P<uint32_t>(w.idx), nt, P<unsigned long long>(w.fpos),
                           tris_dev, st);
        cudaError_t se = cudaGetLastError();
        if (se == cudaSuccess) se = cudaStreamSynchronize(st);
        if (se != cudaSuccess) {
            cudaFree(tris_dev);
            return e.set(GBSDF_ECUDA, "triangle build: %s", cudaGetErrorString(se));
        }
    }
    o.tris_on_device = 1;
    int rc = compute(tris_dev, kept, true, voxel_size, min_coord, max_coord, out, out_on_device != 0, o, stats, e);
    cudaFree(tris_dev);
    return rc;
}

int gbsdf_brick_features(const gbsdf_tri* tris, int64_t n_tris, float voxel_size, const int32_t min_coord[3],
                         const int32_t max_coord[3], int32_t tris_on_device, float* features_dev,
                         int64_t capacity_bricks, int32_t n_bricks[3], char* err, size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!tris || n_tris <= 0 || !min_coord || !max_coord || !features_dev)
        return e.set(GBSDF_EINVAL, "bad arguments");
    long long dims[3];
    for (int k = 0; k < 3; ++k) dims[k] = (long long)max_coord[k] - min_coord[k] + 1;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return e.set(GBSDF_EINVAL, "empty lattice");
    Lattice L = make_lattice(min_coord, max_coord, voxel_size);
    if (n_bricks)
        for (int k = 0; k < 3; ++k) n_bricks[k] = L.nb[k];
    if (L.nbricks > capacity_bricks) return e.set(GBSDF_EINVAL, "feature buffer holds %lld bricks, need %lld",
                                                  (long long)capacity_bricks, L.nbricks);
    // The features are computed on the device that holds features_dev; device triangles
    // must live on that device too.
    int device = 0;
    {
        cudaPointerAttributes fa{};
        if (cudaPointerGetAttributes(&fa, features_dev) != cudaSuccess || fa.type != cudaMemoryTypeDevice) {
            cudaGetLastError();
            return e.set(GBSDF_EINVAL, "features_dev is not device memory");
        }
        device = fa.device;
        if (tris_on_device) {
            cudaPointerAttributes ta{};
            if (cudaPointerGetAttributes(&ta, tris) != cudaSuccess || ta.type != cudaMemoryTypeDevice ||
                ta.device != device) {
                cudaGetLastError();
                return e.set(GBSDF_EINVAL, "device triangles must be on the device of features_dev (%d)", device);
            }
        }
    }
    if (device < 0 || device >= 64) return e.set(GBSDF_ENODEV, "device %d out of range", device);
    gbsdf_options o;
    gbsdf_default_options(&o);
    o.mode = GBSDF_MODE_REFERENCE;
    o.tris_on_device = tris_on_device;
    o.device = device;
    Workspace* wp;
    {
        std::lock_guard<std::mutex> g(g_ws_mu);
        wp = &g_ws[device];
    }
    Workspace& w = *wp;
    std::lock_guard<std::mutex> lk(w.mu);
    int rc = init_ws(w, device, e);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaSetDevice(device));
    GB_CK(ensure(w.t12, (size_t)n_tris * 48));
    GB_CK(cudaMemcpyAsync(w.t12.p, tris, (size_t)n_tris * 48,
                          tris_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, w.st));
    GB_CK(cudaEventRecord(w.ev[0], w.st));
    GB_CK(cudaEventRecord(w.ev[1], w.st));
    return run_fast(w, n_tris, L, o, nullptr, true, nullptr, e, features_dev);
}

// The workspace of `device` for the MLP entry points; the caller takes its lock and then
// calls init_ws under it, as compute() does.
static Workspace* mlp_ws(int32_t device, Err& e, int& rc) {
    rc = GBSDF_OK;
    if (device < 0 || device >= 64) {
        rc = e.set(GBSDF_ENODEV, "device %d out of range", device);
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_ws_mu);
    return &g_ws[device];
}

int gbsdf_mlp_forward(const float* params_dev, const float* features_dev, int64_t n, float* logits_dev,
                      int32_t device, char* err, size_t errlen) {
    Err e{err, errlen};
    if (!params_dev || !features_dev || !logits_dev || n < 0) return e.set(GBSDF_EINVAL, "bad arguments");
    int rc;
    Workspace* w = mlp_ws(device, e, rc);
    if (!w) return rc;
    std::lock_guard<std::mutex> lk(w->mu);
    rc = init_ws(*w, device, e);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaSetDevice(device));
    launch_mlp_forward(params_dev, features_dev, n, logits_dev, w->st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaStreamSynchronize(w->st));
    return GBSDF_OK;
}

int gbsdf_mlp_backward(const float* params_dev, const float* features_dev, const float* labels_dev,
                       const float* weights_dev, int64_t n, float* grad_dev, float* loss_dev, int32_t device,
                       char* err, size_t errlen) {
    Err e{err, errlen};
    if (!params_dev || !features_dev || !labels_dev || !grad_dev || !loss_dev || n <= 0)
        return e.set(GBSDF_EINVAL, "bad arguments");
    int rc;
    Workspace* w = mlp_ws(device, e, rc);
    if (!w) return rc;
    std::lock_guard<std::mutex> lk(w->mu);
    rc = init_ws(*w, device, e);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaSetDevice(device));
    const int parts = mlp_backward_parts(n);
    GB_CK(ensure(w->mparts, (size_t)parts * kMlpParams * 4));
    GB_CK(ensure(w->mlossp, (size_t)parts * 4));
    launch_mlp_backward(params_dev, features_dev, labels_dev, weights_dev, n, P<float>(w->mparts), P<float>(w->mlossp),
                        grad_dev, loss_dev, w->st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaStreamSynchronize(w->st));
    return GBSDF_OK;
}

int gbsdf_mlp_adam(float* params_dev, const float* grad_dev, float* m_dev, float* v_dev, float lr, float beta1,
                   float beta2, float eps, float grad_scale, int32_t step, int32_t device, char* err, size_t errlen) {
    Err e{err, errlen};
    if (!params_dev || !grad_dev || !m_dev || !v_dev || step < 1) return e.set(GBSDF_EINVAL, "bad arguments");
    int rc;
    Workspace* w = mlp_ws(device, e, rc);
    if (!w) return rc;
    std::lock_guard<std::mutex> lk(w->mu);
    rc = init_ws(*w, device, e);
    if (rc != GBSDF_OK) return rc;
    GB_CK(cudaSetDevice(device));
    launch_adam(params_dev, grad_dev, m_dev, v_dev, kMlpParams, lr, beta1, beta2, eps, grad_scale, step, w->st);
    GB_CK(cudaGetLastError());
    GB_CK(cudaStreamSynchronize(w->st));
    return GBSDF_OK;
}

void gbsdf_release_workspace(int32_t device) {
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> g(g_ws_mu);
    std::lock_guard<std::mutex> lk(g_ws[device].mu);
    free_ws(g_ws[device]);
    release_iso_workspace(device);
}

int gbsdf_selftest(int32_t which, int32_t device, uint64_t* result, char* err, size_t errlen) {
    Err e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!result) return e.set(GBSDF_EINVAL, "null result");
    if (which < 0 || which > 2) return e.set(GBSDF_EINVAL, "unknown self-test %d", which);
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device %d", device);
    }
    GB_CK(cudaSetDevice(device));
    unsigned long long* d = nullptr;
    GB_CK(cudaMalloc(&d, sizeof(unsigned long long)));
    cudaError_t rc = cudaMemset(d, 0, sizeof(unsigned long long));
    if (rc == cudaSuccess) {
        if (which == 0 || which == 2) {
            if (which == 0) launch_selftest_div3(d, 0);
            else launch_selftest_godunov(d, 0);
            rc = cudaGetLastError();
        } else if (selftest_tma_tile(d) != 0) {
            cudaFree(d);
            return e.set(GBSDF_ECUDA, "TMA tile self-test could not run (no tensor-map encoder or copy failed)");
        }
    }
    unsigned long long h = 0;
    if (rc == cudaSuccess) rc = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (rc != cudaSuccess) return e.set(GBSDF_ECUDA, "self-test: %s", cudaGetErrorString(rc));
    *result = h;
    return GBSDF_OK;
}

const char* gbsdf_version(void) { return "gbsdf 0.1 (sm_103a)"; }

}  // extern "C"
