// gbsdf_internal.h — host-side declarations shared by the engine's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
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
};

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
    unsigned long long band_voxels;
    unsigned long long splat_evals;    // exact point-triangle evaluations
    unsigned long long unknown_columns;
    unsigned long long listed;         // voxels listed for an exact winding evaluation
    unsigned long long list_overflow;
    unsigned long long fixup_voxels;
    unsigned long long gwn_pairs;      // point-triangle solid-angle evaluations (FP32)
    unsigned long long recheck_n;      // entries in the FP64 re-check list
    unsigned long long fp64_rechecks;  // cumulative
    unsigned long long far_residual;
    unsigned long long safe_clamped;
    unsigned long long patched_voxels;
    int changed[64];                   // per eikonal round
    int stop;                          // eikonal converged flag
    int rounds;
    int verify_state;                  // 0 running, 1 clean, 2 diverged
    int patching;                      // 1 while a patch round is in flight
    int probes;
    int probe_m;                       // mismatches of the current probe
    int total_sites;
    int patch_rounds;
    long long sites[4096];
};

// Consumers of an exact winding decision.
enum GwnConsumer : int { kGwnFixup = 0, kGwnVerify = 1 };

// Kernel launches issued by this library (all launchers count themselves).
unsigned long long& launch_counter();
#define GBSDF_COUNT_LAUNCH() (++::gbsdf::launch_counter())

// ---- launchers (each enqueues on `st`) ------------------------------------------
void launch_prep(const float* tris12, long long T, const Lattice& L, SplatTri* st_out, ParTri* pt_out,
                 unsigned* brick_count, unsigned* strip_count, DevState* ds, cudaStream_t st);
void launch_exclusive_scan(const unsigned* in, unsigned long long* out, long long n, unsigned long long* tmp,
                           long long tmp_elems, cudaStream_t st);
long long scan_tmp_elems(long long n);
void launch_bin_fill(const SplatTri* stt, const ParTri* ptt, long long T, const Lattice& L,
                     const unsigned long long* brick_off, unsigned* brick_cur, unsigned* brick_list,
                     const unsigned long long* strip_off, unsigned* strip_cur, unsigned* strip_list,
                     cudaStream_t st);
void launch_active_bricks(const unsigned* brick_count, long long nbricks, unsigned* active, DevState* ds,
                          cudaStream_t st);
void launch_fill(float* g, long long n, float value, cudaStream_t st);
void launch_splat(const SplatTri* stt, const unsigned long long* brick_off, const unsigned* brick_count,
                  const unsigned* brick_list, const unsigned* active, long long n_active, const Lattice& L,
                  float* dist, DevState* ds, cudaStream_t st);
void launch_parity(const ParTri* ptt, const unsigned long long* strip_off, const unsigned* strip_count,
                   const unsigned* strip_list, const Lattice& L, uint32_t* sbits, uint32_t* ubits, DevState* ds,
                   int signed_crossings, cudaStream_t st);
void launch_list_unknown(uint32_t* ubits, uint32_t* sbits, const Lattice& L, long long* list, long long cap,
                         DevState* ds, int only_if_patching, cudaStream_t st);
// `dist`: the voxel distance field (squared when dist_sq): voxels within
// kSurfaceTolVoxels of the surface are decided inside without a winding sum.
void launch_gwn(const float* tri9, long long T, const Lattice& L, const long long* list, long long list_cap,
                int consumer, int only_if, uint32_t* sbits, long long* recheck, long long recheck_cap,
                const float* dist, int dist_sq, float surf_tol_vox, DevState* ds, int num_sms, cudaStream_t st);
void launch_gwn_recheck(const float* tri9, long long T, const Lattice& L, const long long* recheck,
                        long long recheck_cap, int consumer, uint32_t* sbits, DevState* ds, int num_sms,
                        cudaStream_t st);
void launch_verify_prepare(const Lattice& L, int gen, const uint32_t* ubits, long long* list, DevState* ds,
                           cudaStream_t st);
void launch_verify_plan(int gen, DevState* ds, cudaStream_t st);
void launch_patch_mark(const Lattice& L, uint32_t* ubits, DevState* ds, cudaStream_t st);
void launch_sweep(int rule, int axis, int dir, int round, const float* src, float* dst, const Lattice& L,
                  DevState* ds, cudaStream_t st);
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
void launch_selftest_div3(unsigned long long* mism, cudaStream_t st);

}  // namespace gbsdf
