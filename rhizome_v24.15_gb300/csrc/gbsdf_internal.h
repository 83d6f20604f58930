// gbsdf_internal.h — host-side declarations shared by the engine's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace gbsdf {

// Lattice description. The value at (x, y, z) is for the world point
// ((mn.x + x) h, (mn.y + y) h, (mn.z + z) h); storage is dense, x fastest
// (cuda_rasterizer.cu:117-118).
struct Lattice {
    int mn[3];
    int dims[3];
    float h;
    long long N;        // voxels
    int wx;             // 32-bit sign words per x-row: ceil(dims[0] / 32)
    long long nwords;   // sign words in the grid: wx * dims[1] * dims[2]
    int nb[3];          // bricks per axis (kBrick)
    long long nbricks;
    int nsx;            // parity strips per row: ceil(dims[0] / kStrip)
    long long nstrips;  // nsx * dims[1]
    int px;             // row pitch (floats) of the distance grid the eikonal sweeps address:
                        // dims[0], or dims[0] rounded up to 8 in the sweeps' padded copies
};

// The lattice as the eikonal sweeps see their padded grid copies: rows of a multiple of 8
// floats, so that every row starts on a 32-byte L2 sector (TMA descriptors need 16-byte
// pitches; a row that starts mid-sector splits each 8-voxel chunk of the x sweep across two
// sectors, and the partly written sectors cost DRAM read-modify-writes: 1.45x the x sweep's
// time on 860-voxel rows). The pad columns are never lattice voxels.
constexpr int kRowQuantum = 8;
inline int padded_pitch(int dx) { return (dx + kRowQuantum - 1) / kRowQuantum * kRowQuantum; }
inline Lattice padded(const Lattice& L) {
    Lattice P = L;
    P.px = padded_pitch(L.dims[0]);
    return P;
}
inline long long padded_voxels(const Lattice& L) { return (long long)padded_pitch(L.dims[0]) * L.dims[1] * L.dims[2]; }

// Per-triangle record of the band splat (96 bytes): vertices, AABB, the
// reference's clamped XY footprint and a conservative z range.
struct SplatTri {
    float v[9];
    float bb[6];  // tx0, tx1, ty0, ty1, tz0, tz1
    int fx0, fx1, fy0, fy1;
    int z0, z1;
    int valid;
    int pad[2];
};
static_assert(sizeof(SplatTri) == 96, "SplatTri layout");

// Per-triangle record of the parity pass (80 bytes).
struct ParTri {
    float xyab[4];  // minx, miny, maxx, maxy
    int sx0, sx1, sy0, sy1;  // supercell range of the reference CSR (cuda_rasterizer.cu:848-856)
    float v[9];
    int pad[3];
};
static_assert(sizeof(ParTri) == 80, "ParTri layout");

// Pipeline state kept in device memory; read back once at the end of a build.
struct DevState {
    unsigned long long brick_pairs;    // (triangle, brick) pairs of the splat
    unsigned long long strip_pairs;    // (triangle, strip) pairs of the parity pass
    unsigned long long csr_entries;    // entries of the reference's supercell CSR (guard)
    unsigned long long invalid_tris;   // non-finite or out-of-range coordinates
    unsigned long long active_bricks;
    unsigned long long dense_bricks;   // bricks with more binned triangles than the dense-splat threshold
    unsigned long long band_voxels;
    unsigned long long splat_evals;    // exact point-triangle evaluations
    unsigned long long unknown_columns;
    unsigned long long unknown_columns_kept;  // learned batches: the reference pass's count
    unsigned long long band_err_bits;  // largest |FP32 - FP64| band distance of the samples (double bits)
    unsigned long long band_err_n;     // band voxels sampled for it
    unsigned long long listed;         // voxels listed for an exact winding evaluation
    unsigned long long list_overflow;
    unsigned long long fixup_voxels;
    unsigned long long gwn_pairs;      // point-triangle solid-angle evaluations (FP32)
    unsigned long long recheck_n;      // entries in the FP64 re-check list
    unsigned long long fp64_rechecks;  // cumulative
    unsigned long long far_residual;
    unsigned long long safe_clamped;
    unsigned long long patched_voxels;
    unsigned long long overflow;       // a list outgrew the capacity planned for it (batches)
    unsigned long long wait_timeouts;  // bounded waits (TMA tiles) that gave up
    unsigned long long fwn_cells;      // clusters of the hierarchical winding evaluation
    unsigned long long fwn_certified;  // voxels whose side the cluster bound decided
    unsigned long long fwn_fallback;   // voxels handed to the exact sum (current pass)
    unsigned long long fwn_fallback_total;
    unsigned long long fwn_supers;     // super-clusters (4^3 cluster cubes) of the first stage
    unsigned long long fwn_fallback2;  // voxels the super-cluster stage left to the cluster stage
    int changed[64];                   // per eikonal round
    int stop;                          // eikonal converged flag
    int rounds;
    int verify_state;                  // 0 running, 1 clean, 2 diverged
    int patching;                      // 1 while a patch round is in flight
    int probes;
    int probe_m;                       // mismatches of the current probe
    int total_sites;
    int patch_rounds;
    unsigned proposed;                 // learned mode: bricks the network proposed
    int prop_cut;                      // learned mode: lowest logit bin proposed (device-side budget)
    int wait_polls;                    // tile-wait limit: 0 default, > 0 that many polls, < 0 none
    int escalated;                     // learned mode: the verify diverged, signs re-decided exactly
    int abort_;                        // batches: the build failed a check, write no output
    long long sites[4096];
};

// Consumers of an exact winding decision.
enum GwnConsumer : int { kGwnFixup = 0, kGwnVerify = 1 };

// Learned sign-risk model: 32 brick features -> 64 -> 64 -> 1.
constexpr int kBrickBase = 8;                 // base quantities per brick
constexpr int kMlpIn = 32, kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;
constexpr int kMlpBwdSamples = 64;            // samples per CTA of the backward pass

// The lattice of [min, max] at voxel size h, with its sign-word, brick and strip counts.
Lattice make_lattice(const int32_t mn[3], const int32_t mx[3], float h);

// Kernel launches issued by this library (all launchers count themselves).
unsigned long long& launch_counter();
#define GBSDF_COUNT_LAUNCH() (++::gbsdf::launch_counter())

// ---- launchers (each enqueues on `st`) ------------------------------------------
void launch_prep(const float* tris12, long long T, const Lattice& L, SplatTri* st_out, ParTri* pt_out,
                 unsigned* brick_count, unsigned* strip_count, DevState* ds, cudaStream_t st);
void launch_exclusive_scan(const unsigned* in, unsigned long long* out, long long n, unsigned long long* tmp,
                           long long tmp_elems, cudaStream_t st);
long long scan_tmp_elems(long long n);
// Frees the iso-surface extractor's cached scratch of `device` (k_iso.cu).
void release_iso_workspace(int device);
// With `ds`, the pair lists are known to hold `cap_b` / `cap_s` entries: when the counts
// of this SDF build exceed them the fill writes nothing and sets ds->overflow (the splat and
// parity passes then skip the build).
void launch_bin_fill(const SplatTri* stt, const ParTri* ptt, long long T, const Lattice& L,
                     const unsigned long long* brick_off, unsigned* brick_cur, unsigned* brick_list,
                     const unsigned long long* strip_off, unsigned* strip_cur, unsigned* strip_list,
                     cudaStream_t st, DevState* ds = nullptr, unsigned long long cap_b = ~0ull,
                     unsigned long long cap_s = ~0ull);
// The bricks with binned triangles: those with at most `dense_cut` from the front of
// `active` (DevState::active_bricks), the others from the back (DevState::dense_bricks).
constexpr unsigned kDenseCutDefault = 256;
void launch_active_bricks(const unsigned* brick_count, long long nbricks, unsigned* active, DevState* ds,
                          cudaStream_t st, unsigned dense_cut);
// The splat's tile cut of a lattice class (device, voxels, triangles; by octave): 0 when not
// yet timed. The first fast-path build of a class times the candidates (engine.cu).
unsigned tuned_dense_cut(int device, const Lattice& L, long long T);
void set_tuned_dense_cut(int device, const Lattice& L, long long T, unsigned cut);
void launch_fill(float* g, long long n, float value, cudaStream_t st);
// n_active < 0: the active-brick count is read on the device (one CTA per brick of the
// lattice is launched and the surplus exits), so the launch needs no host round trip.
// The band splat's error against FP64: kBandErrSamples voxels, one per equal stratum of
// the lattice at a fixed golden-ratio offset; those in the band (splat value <= 8h) get the FP64 distance to their
// brick's binned triangles (the splat's own candidates) and the largest difference, in
// voxels, goes to DevState::band_err_bits / band_err_n.
constexpr long long kBandErrSamples = 16384;
void launch_band_error(const SplatTri* stt, const unsigned long long* brick_off, const unsigned* brick_count,
                       const unsigned* brick_list, const Lattice& L, const float* dist, DevState* ds, cudaStream_t st);
// n_active / n_dense: the sparse / dense brick counts (< 0: read on the device, one CTA per
// brick of the lattice launched and the surplus exits).
void launch_splat(const SplatTri* stt, const unsigned long long* brick_off, const unsigned* brick_count,
                  const unsigned* brick_list, const unsigned* active, long long n_active, long long n_dense,
                  const Lattice& L, float* dist, DevState* ds, cudaStream_t st);
void launch_parity(const ParTri* ptt, const unsigned long long* strip_off, const unsigned* strip_count,
                   const unsigned* strip_list, const Lattice& L, uint32_t* sbits, uint32_t* ubits, DevState* ds,
                   int signed_crossings, cudaStream_t st);
// Lists the voxels whose U bit is set, clears their U and S bits and, when `ebits` is
// given, records them there as decided by the exact winding number.
void launch_list_unknown(uint32_t* ubits, uint32_t* sbits, const Lattice& L, long long* list, long long cap,
                         DevState* ds, int only_if_patching, cudaStream_t st, uint32_t* ebits = nullptr);
// `dist`: the voxel distance field (squared when dist_sq): voxels within
// kSurfaceTolVoxels of the surface are decided inside without a winding sum.
void launch_gwn(const float* tri9, long long T, const Lattice& L, const long long* list, long long list_cap,
                int consumer, int only_if, uint32_t* sbits, long long* recheck, long long recheck_cap,
                const float* dist, int dist_sq, float surf_tol_vox, DevState* ds, int num_sms, cudaStream_t st);
// Persistent exact-winding pass over a device-sized list, 32 threads per voxel (any list
// length, no host round trip); `only_if`: skip unless a patch round is in flight.
void launch_gwn_team(const float* tri9, long long T, const Lattice& L, long long* list, long long list_cap,
                     int consumer, uint32_t* sbits, long long* recheck, long long recheck_cap, const float* dist,
                     int dist_sq, float surf_tol_vox, DevState* ds, int num_sms, cudaStream_t st, int only_if = 0);

// ---- hierarchical winding numbers --------------------------------------------------
// Triangles clustered by the grid cube of their centroid; each cluster keeps its
// area-weighted centroid c, area vector D = sum(a_i n_i), first moment M = sum(a_i n_i
// (g_i - c)^T) (g_i the triangle centroids; exact for flat triangles), area A and radius r
// (every vertex within r of c). Seen from q at distance d > beta r, with y = c - q, the
// kernel K(x) = (x - q) / |x - q|^3 expanded to second order gives the cluster's solid
// angle D . y / d^3 + (tr M - 3 y^T M y / d^2) / d^3 within 3 r^2 A / (d - r)^4 (the second
// derivative of K has norm at most 6 / |x - q|^4); nearer clusters are summed exactly. A voxel whose |w| clears 0.5
// by more than the summed bound (plus rounding slack) is decided; the others go to the
// exact per-triangle sum. Decisions therefore equal the exact path's.
struct FwnCell {
    float cx, cy, cz, r;      // centroid, radius
    float ax, ay, az, area;   // area vector, area
    float m[9];               // first moment sum_t D_t,i (g_t - c)_j, row-major (i, j)
    unsigned off, cnt, pad0;
};
static_assert(sizeof(FwnCell) == 80, "FwnCell layout");
// The cluster grid: cubes of s voxels (s = 8, halved down to 2 while the triangles would
// average more than 16 per cube), covering the lattice; triangles are binned by centroid
// (clamped to the grid).
struct FwnGrid {
    int s;
    int n[3];
    long long cells;
};
FwnGrid fwn_grid(const Lattice& L, long long T);
struct Fwn {
    FwnGrid g;
    FwnCell* cells;           // capacity: min(grid cells, triangles)
    unsigned* tri;            // triangles by cluster
    unsigned* cell_of;        // cluster brick of each triangle
    unsigned* counts;         // per grid cell
    unsigned* cursor;         // per grid cell
    unsigned* flag;           // per grid cell: non-empty
    unsigned long long* off;  // per grid cell
    unsigned long long* cidx; // per grid cell: cluster index
    unsigned long long* scan; // scan scratch
    long long* fb;            // voxels left to the exact sum
    long long fb_cap;
    // super-clusters: the clusters of each cube of 4^3 cluster cubes, with aggregated
    // moments; a first query stage uses them for far super-clusters and hands the voxels
    // it cannot decide to the cluster stage (fb2)
    long long scells = 0;            // super grid cubes
    int sn[3] = {0, 0, 0};
    FwnCell* supers = nullptr;       // capacity: min(super cubes, clusters)
    unsigned* sup_of = nullptr;      // per cluster: its super cube
    unsigned* sup_counts = nullptr;  // per super cube
    unsigned* sup_cursor = nullptr;
    unsigned* sup_flag = nullptr;
    unsigned long long* sup_off = nullptr;
    unsigned long long* sup_cidx = nullptr;
    unsigned* sup_child = nullptr;   // clusters by super cube, ascending within a cube
    long long* fb2 = nullptr;        // voxels left to the cluster stage (capacity fb_cap)
};
long long fwn_scan_elems(const FwnGrid& g);
// Bytes of the super-cluster arrays of `g` (T triangles, list capacity `cap`), and their
// carving from one 256-byte aligned allocation into f (sets scells, sn and the pointers).
size_t fwn_super_bytes(const FwnGrid& g, long long T, long long cap);
void fwn_super_carve(Fwn& f, void* base, long long T, long long cap);
// Builds the clusters of the packed triangles (device only, no host round trip).
void launch_fwn_build(const float* tri9, long long T, const Lattice& L, const Fwn& f, DevState* ds, cudaStream_t st);
// Decides the listed voxels (as launch_gwn does) by the cluster bound, then sums the rest
// exactly; the FP64 re-check pass (launch_gwn_recheck) follows as after launch_gwn.
void launch_winding(const Fwn* f, const float* tri9, long long T, const Lattice& L, const long long* list,
                    long long list_cap, int consumer, int only_if, uint32_t* sbits, long long* recheck,
                    long long recheck_cap, const float* dist, int dist_sq, float surf_tol_vox, DevState* ds,
                    int num_sms, cudaStream_t st);
// Batches: decides on the device whether the build passed its checks (valid triangles,
// the reference's CSR guard when `csr_guard`, no list overflow); sets ds->abort_ if not.
void launch_batch_finalize(DevState* ds, int csr_guard, cudaStream_t st);
void launch_gwn_recheck(const float* tri9, long long T, const Lattice& L, long long* recheck,
                        long long recheck_cap, int consumer, uint32_t* sbits, DevState* ds, int num_sms,
                        cudaStream_t st);
void launch_verify_prepare(const Lattice& L, int gen, const uint32_t* ubits, long long* list, DevState* ds,
                           cudaStream_t st);
// escalate (learned mode): any mismatch of a probe ends the verify as diverged, with no
// patch boxes, so the signs are re-decided (launch_escalate) instead.
void launch_verify_plan(int gen, DevState* ds, cudaStream_t st, int escalate = 0);
void launch_patch_mark(const Lattice& L, uint32_t* ubits, DevState* ds, cudaStream_t st);
// TMA descriptor of one grid copy (x fastest) for the staged x sweep. `valid` is false
// when the lattice does not admit one (row pitch not a multiple of 16 bytes) or the
// driver's encoder is unavailable; the x sweep then stages with cp.async.
struct GridMap {
    CUtensorMap map;   // x sweep tile: 8 (x) x 34 (y) x 10 (z), 32-byte swizzle
    CUtensorMap ymap;  // y walk batch: 40 (x) x 4 (y slices) x 18 (z rows)
    CUtensorMap zmap;  // z walk batch: 40 (x) x 18 (y rows) x 4 (z slices)
    CUtensorMap wmap;  // wide x sweep tile: 20 (x) x 34 (y) x 10 (z), no swizzle
    bool valid;
    bool walk_valid;
    bool wide_valid;
};
bool encode_grid_map(GridMap& m, const float* base, const Lattice& L);  // rows L.px floats apart
// The eikonal's padded grid copy: `P` = padded(L); pad writes every element of the copy.
void launch_pad_rows(const float* dense, float* pad, const Lattice& P, cudaStream_t st);
// audit_ds: also count the voxels still at the far sentinel into audit_ds->far_residual (the
// audit, launch_audit, folded into the copy); null: copy only.
void launch_unpad_rows(const float* pad, float* dense, const Lattice& P, cudaStream_t st, DevState* audit_ds);
// Schedules of the x sweep (all give identical results): staged by per-thread cp.async
// copies, by TMA tiles on a CTA-barrier ring, by TMA tiles on a warp-specialised mbarrier
// pipeline, the same pipeline with two lines per thread updated in packed FP32 pairs (the
// reference's update on lattices with at least two voxels along y and z; elsewhere it runs
// as the pipeline), or the pipeline with 16-voxel chunks staged as 20-column boxes (one
// copy per chunk carries its downstream neighbour). 0 picks the pipeline when a TMA
// descriptor is valid.
enum XSchedule : int { kXAuto = 0, kXCpAsync = 1, kXTmaRing = 2, kXTmaPipe = 3, kXTmaPipe2 = 4, kXTmaWide = 5 };
// Schedules of the y and z walks: cp.async slice ring, TMA batches on a warp-specialised
// mbarrier pipeline (one line per thread in two rows, or four adjacent lines per thread,
// or four adjacent lines per thread updated in packed FP32 pairs -- the reference's
// update on lattices with at least two rows across the walk; elsewhere it runs as the
// four-lines schedule). 0 picks the pipeline when its descriptors are valid.
enum WSchedule : int { kWAuto = 0, kWCpAsync = 1, kWTmaPipe = 2, kWTmaVec = 3, kWTmaVec2 = 4 };
// `src_map`: the descriptor of `src` (or null); `x_schedule`: an XSchedule.
void launch_sweep(int rule, int axis, int dir, int round, const float* src, float* dst, const Lattice& L,
                  DevState* ds, cudaStream_t st, const GridMap* src_map = nullptr, int x_schedule = kXAuto,
                  int w_schedule = kWAuto);
// The sweep schedules for this lattice class and phase (0: the first round, 1: later
// rounds): the remembered winners, else (measure) each candidate timed on src -> dst
// (writes dst and changed[63]), else the pipelines.
struct SweepPlan {
    int x;  // XSchedule
    int w;  // WSchedule
};
SweepPlan tuned_sweep_plan(int device, const Lattice& L, const float* src, float* dst, const GridMap* src_map,
                           DevState* ds, cudaStream_t st, bool measure, int phase);
// Layout check of the x sweep's TMA tile (swizzled rows, out-of-lattice fill): writes the
// number of mismatching elements to *mism.
int selftest_tma_tile(unsigned long long* mism);
void launch_end_round(int slot, int round, int cap, DevState* ds, cudaStream_t st);
void launch_audit(const float* g, const Lattice& L, DevState* ds, cudaStream_t st);
void launch_clamp(float* g, const uint32_t* sbits, const Lattice& L, DevState* ds, cudaStream_t st);
void launch_apply(const float* g, const uint32_t* sbits, const Lattice& L, float* out, const DevState* ds,
                  float surf_tol, cudaStream_t st);
void launch_pack_tri9(const float* tris12, long long T, float* tri9, cudaStream_t st);
void launch_gwn_small(const float* tri9, long long T, const Lattice& L, const long long* list, long long list_cap,
                      int consumer, uint32_t* sbits, long long* recheck, long long recheck_cap, const float* dist,
                      int dist_sq, float surf_tol_vox, DevState* ds, long long n_hint, cudaStream_t st);
void launch_tri_flags(const float* verts, long long nv, const uint32_t* idx, long long nt, unsigned* flags,
                      cudaStream_t st);
void launch_tri_scatter(const float* verts, long long nv, const uint32_t* idx, long long nt,
                        const unsigned long long* pos, float* out, cudaStream_t st);
void launch_tile_bounds(const float* t12, long long T, float* hb, cudaStream_t st);
void launch_legacy_dist(const float* t9, long long T, const float* hb, const Lattice& L, float* d2,
                        cudaStream_t st);
void launch_legacy_combine(const float* d2, const uint32_t* sbits, const Lattice& L, float* out, cudaStream_t st);
void launch_iota(long long* list, long long n, long long from, cudaStream_t st);
long long edge_table_cap(long long T);
void launch_open_edges(const float* t12, long long T, const Lattice& L, unsigned long long* keys, unsigned* counts,
                       long long cap, unsigned* open_count, cudaStream_t st);
void launch_brick_features(const float* dist, const uint32_t* S, const uint32_t* E, const uint32_t* S2,
                           const uint32_t* U2, const unsigned* brick_tris, const unsigned* open_count,
                           const Lattice& L, float* base, float* X, cudaStream_t st);
void launch_mlp_forward(const float* P, const float* X, long long B, float* logits, cudaStream_t st);
int mlp_backward_parts(long long B);
void launch_mlp_backward(const float* P, const float* X, const float* y, const float* wt, long long B, float* partial,
                         float* loss_partial, float* grad, float* loss, cudaStream_t st);
void launch_adam(float* P, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                 float scale, int step, cudaStream_t st);
// learned proposals: logit histogram (kPropBins bins above the threshold), the cut bin
// that keeps the proposal count within the budget, then the marking pass
constexpr int kPropBins = 4096;
constexpr float kPropScale = 128.0f;
void launch_propose_hist(const float* logits, long long nb, float logit_thr, unsigned* hist, cudaStream_t st);
// Proposals with the budget's cut taken on the device (no host round trip): the bricks above
// the logit threshold, the highest-scoring ones first, at most `budget` of them, marked
// unknown in U (hist: kPropBins scratch counters); none after an escalation.
void launch_propose_dev(const float* logits, const Lattice& L, float logit_thr, unsigned budget, unsigned* hist,
                        DevState* ds, uint32_t* U, cudaStream_t st);
// Learned mode: when the verify diverged, take the signed-crossing pass's signs (S2) and
// unknown columns (U2) in place of S / U and mark the state clean and escalated.
void launch_escalate(DevState* ds, uint32_t* S, uint32_t* U, const uint32_t* S2, const uint32_t* U2,
                     const Lattice& L, int num_sms, cudaStream_t st);

void launch_selftest_div3(unsigned long long* mism, cudaStream_t st);
void launch_selftest_godunov(unsigned long long* mism, cudaStream_t st);

}  // namespace gbsdf
